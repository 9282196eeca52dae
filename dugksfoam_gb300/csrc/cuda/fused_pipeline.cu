// Fused tile-sweep pipeline (placeholder until the tiled kernels land).
#include "fused.h"

namespace dugks {

std::unique_ptr<FusedPipeline> make_fused_pipeline(Solver&, const StepArgs&, int, std::string& err) {
    err = "fused pipeline not available in this build";
    return nullptr;
}

}  // namespace dugks
