// Fused sweeps in plain FP64 (built without FMA contraction).
#include "fused_pipeline_impl.cuh"

namespace dugks {

std::unique_ptr<FusedPipeline> make_fused_fp64(Solver& s, const StepArgs& a, std::string& err) {
    std::unique_ptr<FusedPipelineT<double>> p(new FusedPipelineT<double>());
    if (!p->init(s, a, err)) return nullptr;
    return p;
}

}  // namespace dugks
