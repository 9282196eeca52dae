// Fused pipeline factory: dispatch on the storage precision.
#include <cstdlib>

#include "dugks/dugks.h"
#include "fused.h"

namespace dugks {

namespace {
thread_local int g_tuneNpl = 0, g_tuneTile = 0;
thread_local bool g_tuneWave = true;
}

void fused_set_tuning(int npl, int maxTileCells, bool waveBalance) {
    g_tuneNpl = npl;
    g_tuneTile = maxTileCells;
    g_tuneWave = waveBalance;
}

int fused_tile_cap() { return g_tuneTile; }
bool fused_wave_balance() { return g_tuneWave && g_tuneTile <= 0; }

int fused_npl(int precision) {
    if (precision == DUGKS_FP64) return 1;
    if (g_tuneNpl == 2 || g_tuneNpl == 4) return g_tuneNpl;
    const char* e = std::getenv("DUGKS_NPL");
    const int npl = e ? std::atoi(e) : 4;
    return (npl == 2 || npl == 4) ? npl : 4;  // packed pairs: an even count per lane
}

bool fused_face_grad() {
    const char* e = std::getenv("DUGKS_FACE_GRAD");
    return e && e[0] == '1';
}

int fused_dv_granule(int precision) { return 32 * fused_npl(precision); }

std::unique_ptr<FusedPipeline> make_fused_pipeline(Solver& s, const StepArgs& a, int precision, std::string& err) {
    return precision == DUGKS_FP64 ? make_fused_fp64(s, a, err) : make_fused_fp32(s, a, err);
}

}  // namespace dugks
