// The reference's exported ISPC kernels (src/ISPC/rayTracerTemplate.ispc),
// batched: one GPU thread per independent call. The reference calls them
// once per node or leaf visit through callIspcTemplateNotConst
// (fastNodeManager.h:306, 396, 788 and the other call sites), passing the
// node's bounds or the leaf block and the FastRay as rayInfo; these kernels
// take arrays of such calls. FastRay records (10 floats: tMax, pos[3],
// invDirection[3], direction[3]; src/fastRay.h:14-29) are used as given:
// the slab test reads invDirection, Moller-Trumbore reads pos and direction.
// Rows are `width` floats long (padding 1, raytracerTemplateGen.py:10).
#include <cuda_runtime.h>

#include "traverse.cuh"

namespace bvhgpu {
namespace dev {

namespace {

BVHGPU_DEV Ray fastray_state(const float* fr) {
  Ray r{};
  r.tmax = fr[0];
  r.o[0] = fr[1]; r.o[1] = fr[2]; r.o[2] = fr[3];
  r.inv[0] = fr[4]; r.inv[1] = fr[5]; r.inv[2] = fr[6];
  r.d[0] = fr[7]; r.d[1] = fr[8]; r.d[2] = fr[9];
  r.exact = true;
  return r;
}

// aabbIntersect{N} (rayTracerTemplate.ispc:171-233): all n lanes, in the
// reference's comparison form; t0 written at hit lanes only.
__global__ void aabb_calls_kernel(int n, const float* __restrict__ bounds,
                                  const uint32_t* __restrict__ offset,
                                  const float* __restrict__ fastrays, float* distances,
                                  uint8_t* result, uint64_t count) {
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const Ray r = fastray_state(fastrays + i * 10);
  const float* bd = bounds + __ldg(offset + i);
  bool any = false;
  for (int j = 0; j < n; ++j) {
    float t0;
    if (slab_dist<false>(bd[j], bd[j + n], bd[j + 2 * n], bd[j + 3 * n], bd[j + 4 * n],
                         bd[j + 5 * n], r, r.tmax, t0)) {
      any = true;
      distances[i * n + j] = t0;
    }
  }
  result[i] = any ? 1 : 0;
}

// triIntersect{L} (rayTracerTemplate.ispc:28-108): lane j % gang keeps its
// first minimum below its running value (initially 1e6); the result is the
// largest index among lanes whose minimum equals the smallest one, and that
// minimum becomes the ray's tMax.
__global__ void tri_calls_kernel(int l, int gang, const float* __restrict__ tri,
                                 const uint32_t* __restrict__ tri_id, float* fastrays,
                                 int32_t* result, uint64_t count) {
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  float* fr = fastrays + i * 10;
  const Ray r = fastray_state(fr);
  const float* blk = tri + __ldg(tri_id + i);
  float t_store[16];
  int orig[16];
  for (int k = 0; k < gang; ++k) {
    t_store[k] = 1000000.0f;
    orig[k] = -1;
  }
  bool any = false;
  for (int j = 0; j < l; ++j) {
    float p[3][3];
    for (int v = 0; v < 3; ++v)
      for (int a = 0; a < 3; ++a) p[v][a] = blk[j + l * (3 * v + a)];
    float t, b1, b2;
    if (moller_trumbore(p, r, r.tmax, t, b1, b2)) {
      const int k = j % gang;
      if (t_store[k] > t) {
        any = true;
        t_store[k] = t;
        orig[k] = j;
      }
    }
  }
  if (!any) {
    result[i] = -1;
    return;
  }
  float best = t_store[0];
  for (int k = 1; k < gang; ++k) best = rmin(best, t_store[k]);
  int idx = -1;
  for (int k = 0; k < gang; ++k)
    if (t_store[k] == best && orig[k] > idx) idx = orig[k];
  fr[0] = best;
  result[i] = idx;
}

// triAnyHit{L} (rayTracerTemplate.ispc:112-168).
__global__ void any_calls_kernel(int l, const float* __restrict__ tri,
                                 const uint32_t* __restrict__ tri_id,
                                 const float* __restrict__ fastrays, uint8_t* result,
                                 uint64_t count) {
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const Ray r = fastray_state(fastrays + i * 10);
  const float* blk = tri + __ldg(tri_id + i);
  uint8_t any = 0;
  for (int j = 0; j < l && !any; ++j) {
    float p[3][3];
    for (int v = 0; v < 3; ++v)
      for (int a = 0; a < 3; ++a) p[v][a] = blk[j + l * (3 * v + a)];
    float t, b1, b2;
    if (moller_trumbore(p, r, r.tmax, t, b1, b2)) any = 1;
  }
  result[i] = any;
}

inline unsigned blocks_for(uint64_t count) { return (unsigned)((count + 127) / 128); }

}  // namespace

cudaError_t launch_aabb_calls(int n, const float* bounds, const uint32_t* offset,
                              const float* fastrays, float* distances, uint8_t* result,
                              uint64_t count, cudaStream_t s) {
  if (count == 0) return cudaSuccess;
  aabb_calls_kernel<<<blocks_for(count), 128, 0, s>>>(n, bounds, offset, fastrays, distances,
                                                       result, count);
  return cudaGetLastError();
}

cudaError_t launch_tri_calls(int l, int gang, const float* tri, const uint32_t* tri_id,
                             float* fastrays, int32_t* result, uint64_t count, cudaStream_t s) {
  if (count == 0) return cudaSuccess;
  tri_calls_kernel<<<blocks_for(count), 128, 0, s>>>(l, gang, tri, tri_id, fastrays, result,
                                                      count);
  return cudaGetLastError();
}

cudaError_t launch_any_calls(int l, const float* tri, const uint32_t* tri_id,
                             const float* fastrays, uint8_t* result, uint64_t count,
                             cudaStream_t s) {
  if (count == 0) return cudaSuccess;
  any_calls_kernel<<<blocks_for(count), 128, 0, s>>>(l, tri, tri_id, fastrays, result, count);
  return cudaGetLastError();
}

}  // namespace dev
}  // namespace bvhgpu
