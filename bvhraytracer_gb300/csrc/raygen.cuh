// Arguments and launchers of the ray-generation kernels (raygen.cu).
#pragma once
#include <cuda_runtime.h>

#include "traverse.cuh"

namespace bvhgpu {
namespace dev {

struct CameraArgs {
  float pos[3];
  float transform[16];  // camera to world, column-major
  uint32_t width, height;
  int workgroup;
  float focal, tmax;
  uint64_t n;           // width * height
};

struct SecondaryArgs {
  const bvhgpu_ray_t* primary;
  const float4* hits;
  uint64_t n;
  const uint32_t* prim_slot;  // input triangle id -> leaf * leaf_memory + lane
  uint32_t n_prims;
  bvhgpu_ray_t* shadow;       // n rays, or null
  bvhgpu_ray_t* ao;           // n * ao_samples rays (hit-major), or null
  float light[3];
  float offset;
  int ao_samples;
  float ao_length;
  int sampling;
  uint64_t seed;
};

cudaError_t launch_camera_rays(const CameraArgs& c, bvhgpu_ray_t* out, cudaStream_t s);
cudaError_t launch_secondary_rays(const SceneDev& sc, const SecondaryArgs& a, cudaStream_t s);
cudaError_t launch_ao_factor(const uint8_t* occluded, uint64_t n, int samples, float* out,
                             cudaStream_t s);

}  // namespace dev
}  // namespace bvhgpu
