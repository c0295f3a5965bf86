// Read-bandwidth probe: the ceiling for kernels whose working set stays in
// L2. The traversal kernels of a scene whose BVH fits the 129 MB L2 read
// their node and leaf bytes from L1 / L2, not HBM, so the HBM copy bandwidth
// is not the bound that applies to them; this kernel measures the L2 read
// rate they can at most reach (a buffer that fits L2, read repeatedly), and,
// with a buffer far larger than L2, the HBM read rate.
#include <cuda_runtime.h>

#include <algorithm>
#include <string>
#include <vector>

#include "bvhgpu_status.hpp"

namespace bvhgpu {
namespace dev {

// Each thread reads 4 x 16 bytes per iteration (four independent loads in
// flight), L2-cached and not L1-cached (ld.global.cg), over `reps` passes of
// the buffer; the XOR of everything read is stored only if it equals an
// improbable value, so the loads cannot be dropped.
__global__ void __launch_bounds__(512) read_stream_kernel(const uint4* __restrict__ p, size_t n16,
                                                          int reps, uint32_t* sink) {
  uint32_t acc = 0;
  const size_t step = (size_t)gridDim.x * blockDim.x;
  const size_t first = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  for (int r = 0; r < reps; ++r) {
    size_t i = first;
    for (; i + 3 * step < n16; i += 4 * step) {
      const uint4 a = __ldcg(p + i), b = __ldcg(p + i + step);
      const uint4 c = __ldcg(p + i + 2 * step), d = __ldcg(p + i + 3 * step);
      acc ^= a.x ^ a.y ^ a.z ^ a.w ^ b.x ^ b.y ^ b.z ^ b.w;
      acc ^= c.x ^ c.y ^ c.z ^ c.w ^ d.x ^ d.y ^ d.z ^ d.w;
    }
    for (; i < n16; i += step) {
      const uint4 a = __ldcg(p + i);
      acc ^= a.x ^ a.y ^ a.z ^ a.w;
    }
  }
  if (acc == 0x9E3779B9u) sink[0] = acc;
}

}  // namespace dev
}  // namespace bvhgpu

using namespace bvhgpu;

extern "C" int bvhgpu_read_bandwidth(int32_t device, uint64_t bytes, int32_t passes,
                                     int32_t repeats, double* gb_per_s) {
  if (!gb_per_s || bytes < 16 * 1024 || passes < 1 || repeats < 1)
    return set_error(BVHGPU_ERR_BAD_ARG, "read bandwidth: bytes >= 16 KiB, passes and repeats >= 1");
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) return set_error(BVHGPU_ERR_NO_DEVICE, "cudaSetDevice failed");
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  const size_t n16 = bytes / 16;
  void* buf = nullptr;
  uint32_t* sink = nullptr;
  cudaEvent_t t0 = nullptr, t1 = nullptr;
  std::vector<float> ms;
  auto fail = [&](cudaError_t err, const char* what) {
    if (t0) cudaEventDestroy(t0);
    if (t1) cudaEventDestroy(t1);
    cudaFree(buf);
    cudaFree(sink);
    return set_error(BVHGPU_ERR_CUDA, std::string("read bandwidth: ") + what + ": " +
                                          cudaGetErrorString(err));
  };
  if ((e = cudaMalloc(&buf, n16 * 16)) != cudaSuccess) return fail(e, "cudaMalloc");
  if ((e = cudaMalloc(&sink, 4)) != cudaSuccess) return fail(e, "cudaMalloc");
  if ((e = cudaMemset(buf, 0x5A, n16 * 16)) != cudaSuccess) return fail(e, "cudaMemset");
  if ((e = cudaEventCreate(&t0)) != cudaSuccess || (e = cudaEventCreate(&t1)) != cudaSuccess)
    return fail(e, "cudaEventCreate");
  const int blocks = std::max(1, sms) * 4;
  const auto* p = static_cast<const uint4*>(buf);
  dev::read_stream_kernel<<<blocks, 512>>>(p, n16, 1, sink);  // brings the buffer into L2
  for (int k = 0; k < repeats; ++k) {
    cudaEventRecord(t0);
    dev::read_stream_kernel<<<blocks, 512>>>(p, n16, passes, sink);
    cudaEventRecord(t1);
    if ((e = cudaEventSynchronize(t1)) != cudaSuccess) return fail(e, "kernel");
    float m = 0.f;
    cudaEventElapsedTime(&m, t0, t1);
    ms.push_back(m);
  }
  if ((e = cudaGetLastError()) != cudaSuccess) return fail(e, "launch");
  std::sort(ms.begin(), ms.end());
  const double med = ms[ms.size() / 2];
  *gb_per_s = (double)n16 * 16.0 * passes / (med * 1e-3) / 1e9;
  cudaEventDestroy(t0);
  cudaEventDestroy(t1);
  cudaFree(buf);
  cudaFree(sink);
  return BVHGPU_OK;
}
