// Q8 node encoding on the device (q8_encode.cu).
#pragma once
#include <cuda_runtime.h>

#include "traverse.cuh"

namespace bvhgpu {
namespace dev {

// Encodes n_nodes FP32 records (layout NodeFmt<nm, FP32>) into Q8 records
// and their push sequences into the Q8 side array (NodeFmt<nm, Q8>::PSB
// bytes per node); records a kDevErrQ8Encode in *status if a decoded box
// would not contain its FP32 box (not expected for finite boxes).
cudaError_t launch_q8_encode(int nm, const uint8_t* fp32_nodes, uint8_t* q8_nodes,
                             uint8_t* q8_perm, uint32_t n_nodes, int* status, cudaStream_t s);

}  // namespace dev
}  // namespace bvhgpu
