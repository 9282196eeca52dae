// Fused pipeline factory: dispatch on the storage precision.
#include <cstdlib>
#include <string>

#include "dugks/dugks.h"
#include "fused.h"

namespace dugks {

int fused_npl(int precision) {
    if (precision == DUGKS_FP64) return 1;
    const char* e = std::getenv("DUGKS_NPL");
    const int npl = e ? std::atoi(e) : 4;
    return (npl == 2 || npl == 4) ? npl : 4;  // packed pairs: an even count per lane
}

int fused_ctas_per_sm() {
    const char* e = std::getenv("DUGKS_CTAS");
    const int c = e ? std::atoi(e) : 1;
    return c == 2 ? 2 : 1;
}

bool fused_cell_gather() {
    const char* e = std::getenv("DUGKS_CELL_SWEEP");
    return !(e && std::string(e) == "tiled");
}

bool fused_face_pipe() {
    const char* e = std::getenv("DUGKS_SWEEPA_PIPE");
    return !(e && std::string(e) == "0");
}

bool fused_face_sides() {
    const char* e = std::getenv("DUGKS_SWEEPA");
    return !(e && std::string(e) == "owned");
}

int fused_dv_granule(int precision) { return 32 * fused_npl(precision); }

std::unique_ptr<FusedPipeline> make_fused_pipeline(Solver& s, const StepArgs& a, int precision, std::string& err) {
    return precision == DUGKS_FP64 ? make_fused_fp64(s, a, err) : make_fused_fp32(s, a, err);
}

}  // namespace dugks
