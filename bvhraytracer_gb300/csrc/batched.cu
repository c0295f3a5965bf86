// Instantiation and launch of the batched (multi-scene) persistent kernel.
#include <cuda_runtime.h>

// Slab tests of the multi-scene kernel: packed pairs (1) or one child per
// instruction (0), independent of the single-scene kernels' choice. Device
// code is compiled per translation unit (no device linking), so the two
// choices do not meet.
#ifndef BVHGPU_BATCHED_PAIRED
#define BVHGPU_BATCHED_PAIRED 0
#endif
#undef BVHGPU_PAIRED_SLABS
#define BVHGPU_PAIRED_SLABS BVHGPU_BATCHED_PAIRED
// The jobs carry no per-child entries: pushes decode the record (entries
// and triangle bounds both in 112-byte job records measured 6.88 against
// 6.20 ms on the 64-scene batch). BVHGPU_BATCHED_BOUNDS 1: the leaf pre-test
// reads the job scene's stored triangle bounds, and any-hit rays run all of
// a leaf's pre-tests before the full tests of the passing triangles; 0: the
// pre-test computes the bounds from the vertices. 64-scene batch, one launch
// per ray kind: 5.77 ms against 6.19 ms (one launch for all jobs: 5.96
// against 6.23 ms).
#ifndef BVHGPU_BATCHED_BOUNDS
#define BVHGPU_BATCHED_BOUNDS 1
#endif
#undef BVHGPU_LEAF_BOUNDS
#define BVHGPU_LEAF_BOUNDS BVHGPU_BATCHED_BOUNDS

#include "batched.cuh"

namespace bvhgpu {
namespace dev {

size_t batched_param_bytes() { return sizeof(JobTable); }

cudaError_t launch_batched(const JobTable& t, int profile, int kmode, int sm_count,
                           cudaStream_t s) {
  const int bs = 128;
  const size_t smem = (size_t)t.stack_cap * bs * 4;
  constexpr int F = BVHGPU_PROFILE_FAST, I = BVHGPU_PROFILE_INSTRUMENTED;
  void (*k)(const JobTable) =
      profile == F ? (kmode == 1   ? trace_batched_kernel<F, 1>
                      : kmode == 2 ? trace_batched_kernel<F, 2>
                      : kmode == 3 ? trace_batched_kernel<F, 3>
                                   : trace_batched_kernel<F, 0>)
                   : (kmode == 1   ? trace_batched_kernel<I, 1>
                      : kmode == 2 ? trace_batched_kernel<I, 2>
                      : kmode == 3 ? trace_batched_kernel<I, 3>
                                   : trace_batched_kernel<I, 0>);
  cudaError_t e = cudaSuccess;
  if (smem > 48 * 1024)
    e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, bs, smem);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) per_sm = 1;
  uint64_t grid = (uint64_t)per_sm * sm_count;
  const uint64_t need = (t.total + bs - 1) / bs;
  if (grid > need) grid = need;
  if (grid == 0) return cudaSuccess;
  e = cudaMemsetAsync(t.head, 0, sizeof(unsigned long long), s);
  if (e != cudaSuccess) return e;
  if (kmode == 3) {
    e = cudaMemsetAsync(t.head_any, 0, sizeof(unsigned long long), s);
    if (e != cudaSuccess) return e;
  }
  k<<<(unsigned)grid, bs, smem, s>>>(t);
  return cudaGetLastError();
}

}  // namespace dev
}  // namespace bvhgpu
