// Ray reordering by direction before a trace (see reorder.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "bvhgpu.h"

namespace bvhgpu {
namespace dev {

constexpr int kReorderMaxK = 32;  // bins per face side: 6 * 32^2 + 1 bins at most

// Device scratch bytes for reordering n rays into 6 k^2 + 1 bins.
size_t reorder_scratch_bytes(uint64_t n, int k);

// Writes into perm[0..n) the input ray indices grouped by direction bin;
// `scratch` holds reorder_scratch_bytes(n, k) bytes (256-byte aligned).
// Asynchronous on s.
cudaError_t reorder_rays(const bvhgpu_ray_t* rays, uint64_t n, int k, uint32_t* perm,
                         void* scratch, cudaStream_t s);

}  // namespace dev
}  // namespace bvhgpu
