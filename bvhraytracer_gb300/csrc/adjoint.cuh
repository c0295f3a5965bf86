// Arguments and launcher of the adjoint kernel (adjoint.cu).
#pragma once
#include <cuda_runtime.h>

#include "traverse.cuh"

namespace bvhgpu {
namespace dev {

struct AdjointArgs {
  const bvhgpu_ray_t* rays;
  uint64_t n;
  const float4* grad_hits;  // per ray: (unused, dL/dt, dL/db1, dL/db2); null: the arrays below
  float* grad_tri9;         // per input triangle: dL/dp0, dL/dp1, dL/dp2 (accumulated)
  float* grad_rays;         // per ray: dL/do (3), 0, dL/dd (3), 0 (written)
  int stack_cap;
  // With faces: the vertex gradients are added into grad_verts[3 * v + axis]
  // for the triangle's vertex ids faces[3 * prim + k] instead of grad_tri9.
  const int32_t* faces = nullptr;
  float* grad_verts = nullptr;
  uint32_t n_verts = 0;     // vertex ids outside [0, n_verts) are skipped and reported
  // Stored closest hits (prim, t, u, v) of the forward pass: no re-trace.
  const float4* hits = nullptr;
  const uint32_t* prim_slot = nullptr;  // input triangle id -> leaf * leaf_memory + lane
  uint32_t n_prims = 0;
  // Without grad_hits: dL/dt, dL/db1, dL/db2 as separate arrays (null: zero).
  const float* grad_t = nullptr;
  const float* grad_u = nullptr;
  const float* grad_v = nullptr;
};

cudaError_t launch_adjoint(const SceneDev& sc, int nm, const AdjointArgs& a, cudaStream_t s);

}  // namespace dev
}  // namespace bvhgpu
