// Host-side launch helpers: pick the kernel instance for a trace request.
#pragma once
#include <cuda_runtime.h>

#include "traverse.cuh"

namespace bvhgpu {
namespace dev {

struct LaunchCfg {
  int kind = BVHGPU_CLOSEST;
  int scheme = BVHGPU_PER_RAY;
  int profile = BVHGPU_PROFILE_INSTRUMENTED;
  bool count = false;
  int block = 128;      // per-ray scheme threads per block
  int packet = 256;     // stream scheme rays per block
  int policy = 0;       // persistent scheme: 0 while-while, 1 if-if, 2 speculative any-hit,
                        // 3 the same with two leaves per lane, 4 as 3 with the leaves
                        // tested warp-wide
  int refill_min = 8;   // persistent scheme: idle lanes that trigger a refill
  unsigned long long* queue = nullptr;  // persistent scheme: queue head
  bool queue_cleared = false;  // true: the caller zeroed the head already
  int sm_count = 152;
  int fmt = BVHGPU_NODES_FP32;  // node record format of the scene
  uint32_t top_nodes = 0;       // persistent scheme: inner records staged in shared memory
  uint32_t stall_bytes = 0;     // failure-detection tests (see bvhgpu_scene_inject_stall)
  bool save_distance = false;   // per-ray scheme: save-distance traversal (closest hits)
  int reorder = 0;              // > 0: group rays into 6 reorder^2 direction bins first
  bool stack_local = false;     // per-ray scheme: stacks in local memory (cap <= kLocalStack)
  bool any_order = false;       // any-hit rays without counters: child-index push order
};

constexpr int kLocalStack = 64;  // entries of the local-memory stack variant

template <typename K>
inline cudaError_t set_smem(K kernel, size_t bytes) {
  if (bytes <= 48 * 1024) return cudaSuccess;
  return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

template <int NM, int PROFILE, int KIND, bool COUNT, int FMT>
inline cudaError_t launch_one(const SceneDev& sc, const TraceArgs& a, const LaunchCfg& cfg,
                              cudaStream_t s) {
  if (a.n == 0) return cudaSuccess;
  if (cfg.scheme == BVHGPU_PER_RAY) {
    const int bs = cfg.block;
    // Any-hit rays never lower tMax, so a pushed entry (t0 <= t1 <= tMax) is
    // never dropped: save-distance any-hit traversal is the plain one.
    constexpr bool kDist = KIND == BVHGPU_CLOSEST;
    const bool dist = kDist && cfg.save_distance;
    const bool local = cfg.stack_local && !dist && !COUNT && a.stack_cap <= kLocalStack;
    const size_t smem = local ? 0 : (size_t)a.stack_cap * bs * 4 * (dist ? 2 : 1);
    auto k = dist ? trace_dfs_kernel<NM, PROFILE, KIND, COUNT, FMT, kDist>
             : local ? trace_dfs_kernel<NM, PROFILE, KIND, COUNT, FMT, false, (COUNT ? 0 : kLocalStack)>
                     : trace_dfs_kernel<NM, PROFILE, KIND, COUNT, FMT, false>;
    cudaError_t e = set_smem(k, smem);
    if (e != cudaSuccess) return e;
    const uint64_t grid = (a.n + bs - 1) / bs;
    k<<<(unsigned)grid, bs, smem, s>>>(sc, a);
  } else if (cfg.scheme == BVHGPU_PERSISTENT) {
    const int bs = 128;
    // Policies 2 to 4 change the order of leaf tests, which only any-hit
    // rays without counters may do; the others fall back to policy 0.
    constexpr bool kSpec = KIND == BVHGPU_ANY && !COUNT;
    const bool coop = cfg.policy == 4 && kSpec;
    const size_t smem = (size_t)a.stack_cap * bs * 4 +
                        ((size_t)cfg.top_nodes * NodeFmt<NM, FMT>::REC + 15) / 16 * 16 +
                        (coop ? (size_t)bs * kRayRecWords * 4 : 0);
    auto k = cfg.policy == 1 ? trace_persistent_kernel<NM, PROFILE, KIND, COUNT, 1, FMT>
             : (cfg.policy == 2 && kSpec)
                 ? trace_persistent_kernel<NM, PROFILE, KIND, COUNT, (kSpec ? 2 : 0), FMT>
             : (cfg.policy == 3 && kSpec)
                 ? trace_persistent_kernel<NM, PROFILE, KIND, COUNT, (kSpec ? 3 : 0), FMT>
             : coop ? trace_persistent_kernel<NM, PROFILE, KIND, COUNT, (kSpec ? 4 : 0), FMT>
                    : trace_persistent_kernel<NM, PROFILE, KIND, COUNT, 0, FMT>;
    cudaError_t e = set_smem(k, smem);
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, bs, smem);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) per_sm = 1;
    uint64_t grid = (uint64_t)per_sm * cfg.sm_count;
    const uint64_t need = (a.n + bs - 1) / bs;
    if (grid > need) grid = need;
    QueueArgs q{cfg.queue, cfg.refill_min, cfg.top_nodes, cfg.top_nodes ? cfg.stall_bytes : 0u};
    if (!cfg.queue_cleared) {
      e = cudaMemsetAsync(cfg.queue, 0, sizeof(unsigned long long), s);
      if (e != cudaSuccess) return e;
    }
    k<<<(unsigned)grid, bs, smem, s>>>(sc, a, q);
  } else {
    if (FMT != kFmtFP32) return cudaErrorNotSupported;
    const int p = cfg.packet;
    const size_t smem = stream_smem_bytes(p, a.stack_cap, COUNT, COUNT && a.step_stats);
    auto k = trace_stream_kernel<NM, PROFILE, KIND, COUNT>;
    cudaError_t e = set_smem(k, smem);
    if (e != cudaSuccess) return e;
    const uint64_t grid = (a.n + p - 1) / p;
    k<<<(unsigned)grid, p, smem, s>>>(sc, a);
  }
  return cudaGetLastError();
}

template <int NM, int PROFILE, int KIND, bool COUNT>
inline cudaError_t launch_fmt(const SceneDev& sc, const TraceArgs& a, const LaunchCfg& c,
                              cudaStream_t s) {
  if (c.fmt == kFmtQ8) return launch_one<NM, PROFILE, KIND, COUNT, kFmtQ8>(sc, a, c, s);
  return launch_one<NM, PROFILE, KIND, COUNT, kFmtFP32>(sc, a, c, s);
}

template <int NM>
inline cudaError_t launch_for_width(const SceneDev& sc, const TraceArgs& a, const LaunchCfg& c,
                                    cudaStream_t s) {
  const int code = (c.profile << 2) | (c.kind << 1) | (c.count ? 1 : 0);
  switch (code) {
    case 0: return launch_fmt<NM, 0, 0, false>(sc, a, c, s);
    case 1: return launch_fmt<NM, 0, 0, true>(sc, a, c, s);
    case 2: return launch_fmt<NM, 0, 1, false>(sc, a, c, s);
    case 3: return launch_fmt<NM, 0, 1, true>(sc, a, c, s);
    case 4: return launch_fmt<NM, 1, 0, false>(sc, a, c, s);
    case 5: return launch_fmt<NM, 1, 0, true>(sc, a, c, s);
    case 6: return launch_fmt<NM, 1, 1, false>(sc, a, c, s);
    case 7: return launch_fmt<NM, 1, 1, true>(sc, a, c, s);
  }
  return cudaErrorInvalidValue;
}

cudaError_t launch_trace_n4(const SceneDev&, const TraceArgs&, const LaunchCfg&, cudaStream_t);
cudaError_t launch_trace_n8(const SceneDev&, const TraceArgs&, const LaunchCfg&, cudaStream_t);
cudaError_t launch_trace_n12(const SceneDev&, const TraceArgs&, const LaunchCfg&, cudaStream_t);
cudaError_t launch_trace_n16(const SceneDev&, const TraceArgs&, const LaunchCfg&, cudaStream_t);

}  // namespace dev
}  // namespace bvhgpu
