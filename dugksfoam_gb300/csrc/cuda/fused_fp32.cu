// Fused sweeps with FP32 distributions (FP64 moments and macros).
#include "fused_pipeline_impl.cuh"

namespace dugks {

std::unique_ptr<FusedPipeline> make_fused_fp32(Solver& s, const StepArgs& a, std::string& err) {
    std::unique_ptr<FusedPipelineT<float>> p(new FusedPipelineT<float>());
    if (!p->init(s, a, err)) return nullptr;
    return p;
}

}  // namespace dugks
