// Fused pipeline factory: dispatch on the storage precision.
#include <cstdlib>

#include "dugks/dugks.h"
#include "fused.h"

namespace dugks {

int fused_dv_granule() {
    const char* e = std::getenv("DUGKS_NPL");
    int npl = e ? std::atoi(e) : 1;
    return 32 * (npl == 2 ? 2 : 1);
}

std::unique_ptr<FusedPipeline> make_fused_pipeline(Solver& s, const StepArgs& a, int precision, std::string& err) {
    return precision == DUGKS_FP64 ? make_fused_fp64(s, a, err) : make_fused_fp32(s, a, err);
}

}  // namespace dugks
