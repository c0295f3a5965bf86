// FP64 check kernel: the closest-hit record of each ray recomputed in double
// precision for the same ray / triangle pair (Moller-Trumbore in FP64), so the
// error of every FP32 result can be stated. This is the only kernel that uses
// FP64 arithmetic apart from the reference's rare edge fallback inside the
// watertight test.
#include <cuda_runtime.h>

#include "traverse.cuh"

namespace bvhgpu {
namespace dev {

struct Fp64Args {
  const bvhgpu_ray_t* rays;
  const float4* hits;
  uint64_t n;
  const uint32_t* prim_slot;  // input triangle id -> leaf * leaf_memory + lane
  uint32_t n_prims;
  int profile;
  double* out;  // per ray: t64, b1_64, b2_64, |t32 - t64| / |t64|
};

__global__ void fp64_check_kernel(SceneDev sc, Fp64Args a) {
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  double* o4 = a.out + i * 4;
  const float4 h = a.hits[i];
  const int prim = __float_as_int(h.x);
  if (prim < 0 || (uint32_t)prim >= a.n_prims) {
    o4[0] = o4[1] = o4[2] = o4[3] = __longlong_as_double(0x7FF8000000000000ll);
    return;
  }
  const uint32_t slot = a.prim_slot[prim];
  const uint32_t leaf = slot / (uint32_t)sc.leaf_memory, lane = slot % (uint32_t)sc.leaf_memory;
  const float* blk = sc.leaves + (size_t)leaf * 9 * sc.leaf_memory;
  int st = sc.leaf_memory;
  if (isnan(blk[sc.leaf_memory * 9 - 1])) st = (int)blk[sc.leaf_memory * 9 - 2];
  double p[3][3];
  for (int v = 0; v < 3; ++v)
    for (int k = 0; k < 3; ++k) p[v][k] = (double)blk[(v * 3 + k) * st + lane];
  const bvhgpu_ray_t in = load_ray(a.rays, i);
  // The FP32 ray the kernels traced (normalised in the instrumented profile).
  const Ray r = a.profile == BVHGPU_PROFILE_FAST ? make_ray<BVHGPU_PROFILE_FAST>(in)
                                                 : make_ray<BVHGPU_PROFILE_INSTRUMENTED>(in);
  const double o[3] = {r.o[0], r.o[1], r.o[2]}, d[3] = {r.d[0], r.d[1], r.d[2]};
  double e1[3], e2[3], s[3];
  for (int k = 0; k < 3; ++k) {
    e1[k] = p[1][k] - p[0][k];
    e2[k] = p[2][k] - p[0][k];
    s[k] = o[k] - p[0][k];
  }
  const double s1[3] = {d[1] * e2[2] - d[2] * e2[1], d[2] * e2[0] - d[0] * e2[2],
                        d[0] * e2[1] - d[1] * e2[0]};
  const double div = s1[0] * e1[0] + s1[1] * e1[1] + s1[2] * e1[2];
  const double inv = 1.0 / div;
  const double b1 = (s[0] * s1[0] + s[1] * s1[1] + s[2] * s1[2]) * inv;
  const double s2[3] = {s[1] * e1[2] - s[2] * e1[1], s[2] * e1[0] - s[0] * e1[2],
                        s[0] * e1[1] - s[1] * e1[0]};
  const double b2 = (d[0] * s2[0] + d[1] * s2[1] + d[2] * s2[2]) * inv;
  const double t = (e2[0] * s2[0] + e2[1] * s2[1] + e2[2] * s2[2]) * inv;
  o4[0] = t;
  o4[1] = b1;
  o4[2] = b2;
  o4[3] = fabs((double)h.y - t) / fabs(t);
}

cudaError_t launch_fp64_check(const SceneDev& sc, const Fp64Args& a, cudaStream_t s) {
  if (a.n == 0) return cudaSuccess;
  const int bs = 256;
  fp64_check_kernel<<<(unsigned)((a.n + bs - 1) / bs), bs, 0, s>>>(sc, a);
  return cudaGetLastError();
}

}  // namespace dev
}  // namespace bvhgpu
