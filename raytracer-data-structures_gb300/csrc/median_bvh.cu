// Median BVH build (constructBVHNew, accelerators.h:246-337) on the GPU.
#include "rq_build.hpp"

namespace rq {

BuildResult build_median_bvh(const SceneView&, AccelBuffers&, BuildScratch&, uint32_t*, cudaStream_t) {
  return BuildResult::error(RQ_ERROR_UNSUPPORTED, "BVH builder not available yet");
}

}  // namespace rq
