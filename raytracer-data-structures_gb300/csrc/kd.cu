// SAH KD-tree build and traversal (accelerators.h:715-1086) on the GPU.
#include "rq_build.hpp"

namespace rq {

BuildResult build_kd_tree(const SceneView&, int, AccelBuffers&, BuildScratch&, uint32_t*, cudaStream_t) {
  return BuildResult::error(RQ_ERROR_UNSUPPORTED, "KD builder not available yet");
}

void launch_trace_kd(int, int, bool, const KdView&, const float4*, uint32_t, float4*, uint32_t*, uint32_t*,
                     cudaStream_t) {}

}  // namespace rq
