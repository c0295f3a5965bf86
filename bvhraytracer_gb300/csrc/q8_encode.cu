// Q8 node encoding on the device: FP32 node records in, Q8 records out, one
// thread per inner node. The arithmetic is that of the host encoder in
// bvh_export.cpp (which stays as the specification): per axis a power-of-two
// step 2^e, the smallest e >= max(-126, exponent of extent / 255) with
// origin + 255 * step >= the node's high bound when rounded up; per child the
// largest q_lo with origin + q_lo * step <= lo rounded down and the smallest
// q_hi with origin + q_hi * step >= hi rounded up. q * step is exact, and the
// directed roundings are __fadd_rd / __fadd_ru, so the records equal the
// host's byte for byte. The meta block is copied, the leaf counts are packed
// as (count - 1) nibbles, and the push sequences go to the Q8 side array.
#include <cuda_runtime.h>

#include "q8_encode.cuh"

namespace bvhgpu {
namespace dev {

namespace {

__device__ __forceinline__ float step_of(int e) {
  // 2^e for -126 <= e <= 127, exactly.
  return __int_as_float((e + 127) << 23);
}

template <int NM>
__global__ void q8_encode_kernel(const uint8_t* __restrict__ in, uint8_t* __restrict__ out,
                                 uint8_t* __restrict__ perm_out, uint32_t n_nodes, int* status) {
  using F32 = NodeFmt<NM, kFmtFP32>;
  using Q8 = NodeFmt<NM, kFmtQ8>;
  const uint32_t node = blockIdx.x * blockDim.x + threadIdx.x;
  if (node >= n_nodes) return;
  const uint8_t* src = in + (size_t)node * F32::REC;
  uint8_t* dst = out + (size_t)node * Q8::REC;
  for (int b = 0; b < Q8::REC; b += 4) *reinterpret_cast<uint32_t*>(dst + b) = 0u;
  const float* box = reinterpret_cast<const float*>(src);
  const int count = (int)src[F32::META + 10];
  // Meta (12 B) copied; leaf counts (NM bytes) packed as (count - 1)
  // nibbles; push sequences (6 words) to the side array.
  for (int b = 0; b < 12; ++b) dst[Q8::META + b] = src[F32::META + b];
  for (int j = 0; j < NM; ++j) {
    const int c = src[F32::LCNT + j];
    if (c > 0) dst[Q8::LCNT + j / 2] |= (uint8_t)(((c - 1) & 15) << (4 * (j & 1)));
  }
  uint8_t* perm = perm_out + (size_t)node * Q8::PSB;
  for (int b = 0; b < Q8::PSB; ++b) perm[b] = src[F32::PERM + b];
  float origin[3];
  int ex[3];
  for (int k = 0; k < 3; ++k) {
    // The node's own box is the union of its children's boxes.
    float lo = box[k * NM], hi = box[(3 + k) * NM];
    for (int j = 1; j < count; ++j) {
      lo = fminf(lo, box[k * NM + j]);
      hi = fmaxf(hi, box[(3 + k) * NM + j]);
    }
    origin[k] = lo;
    const float ext = hi - lo;
    int e = -126;
    if (ext > 0.0f) {
      int fe;
      frexp((double)ext / 255.0, &fe);
      e = max(-126, fe - 1);
    }
    while (e < 127 && __fadd_ru(origin[k], 255.0f * step_of(e)) < hi) ++e;
    ex[k] = e;
  }
  float* o = reinterpret_cast<float*>(dst);
  o[0] = origin[0];
  o[1] = origin[1];
  o[2] = origin[2];
  dst[12] = (uint8_t)(int8_t)ex[0];
  dst[13] = (uint8_t)(int8_t)ex[1];
  dst[14] = (uint8_t)(int8_t)ex[2];
  uint8_t* q = dst + Q8::QBOX;
  for (int j = 0; j < count; ++j) {
    for (int k = 0; k < 3; ++k) {
      const float step = step_of(ex[k]);
      const float lo = box[k * NM + j], hi = box[(3 + k) * NM + j];
      const double fl = floor(((double)lo - (double)origin[k]) / (double)step);
      int ql = (int)fmin(255.0, fmax(0.0, fl));
      while (ql > 0 && __fadd_rd(origin[k], (float)ql * step) > lo) --ql;
      while (ql < 255 && __fadd_rd(origin[k], (float)(ql + 1) * step) <= lo) ++ql;
      const double ce = ceil(((double)hi - (double)origin[k]) / (double)step);
      int qh = (int)fmin(255.0, fmax(0.0, ce));
      while (qh < 255 && __fadd_ru(origin[k], (float)qh * step) < hi) ++qh;
      while (qh > 0 && __fadd_ru(origin[k], (float)(qh - 1) * step) >= hi) --qh;
      if (__fadd_rd(origin[k], (float)ql * step) > lo || __fadd_ru(origin[k], (float)qh * step) < hi)
        atomicCAS(status, 0, kDevErrQ8Encode);
      q[k * NM + j] = (uint8_t)ql;
      q[(3 + k) * NM + j] = (uint8_t)qh;
    }
  }
}

}  // namespace

cudaError_t launch_q8_encode(int nm, const uint8_t* fp32_nodes, uint8_t* q8_nodes,
                             uint8_t* q8_perm, uint32_t n_nodes, int* status, cudaStream_t s) {
  if (n_nodes == 0) return cudaSuccess;
  const unsigned grid = (n_nodes + 127) / 128;
  switch (nm) {
    case 4: q8_encode_kernel<4><<<grid, 128, 0, s>>>(fp32_nodes, q8_nodes, q8_perm, n_nodes, status); break;
    case 8: q8_encode_kernel<8><<<grid, 128, 0, s>>>(fp32_nodes, q8_nodes, q8_perm, n_nodes, status); break;
    case 12: q8_encode_kernel<12><<<grid, 128, 0, s>>>(fp32_nodes, q8_nodes, q8_perm, n_nodes, status); break;
    case 16: q8_encode_kernel<16><<<grid, 128, 0, s>>>(fp32_nodes, q8_nodes, q8_perm, n_nodes, status); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

}  // namespace dev
}  // namespace bvhgpu
