// Kernel instantiations for node records with 8 child slots.
#include "launch.cuh"

namespace bvhgpu {
namespace dev {
cudaError_t launch_trace_n8(const SceneDev& sc, const TraceArgs& a, const LaunchCfg& cfg,
                              cudaStream_t s) {
  return launch_for_width<8>(sc, a, cfg, s);
}
}  // namespace dev
}  // namespace bvhgpu
