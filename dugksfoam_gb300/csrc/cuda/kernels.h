// Host-callable launchers of the DUGKS CUDA kernels.
#pragma once

#include <cuda_runtime.h>

#include "device_common.cuh"

namespace dugks {

// ---------------------------------------------------------- reference pipeline
constexpr int kRefKernels = 8;
extern const char* const kRefKernelNames[kRefKernels];

struct RefBuffers {
    double *gT, *hT;     // [nC][Vp]      g~, h~
    double *gB, *hB;     // [nC][Vp]      gBarPvol, hBarPvol
    double *gG, *hG;     // [nC][D][Vp]   least-squares gradients
    double *Gbg, *Gbh;   // [nW][Vp]      lagged fixedGradient gradients
    double *gS, *hS;     // [nA][Vp]      face distributions
    double *gSym, *hSym; // [nW][Vp]      snapshot of symmetry faces (when present)
};

// Launch pass `pass` (0..kRefKernels-1) of one reference-pipeline step.
// Pass 3 also runs the symmetry-patch copy, pass 7 the pressure-patch update.
void launch_ref_pass(int pass, const StepArgs& a, const RefBuffers& b, int sms, cudaStream_t s);
// P10 update of pressureIn / pressureOut patch values from the cell macros in a.
void launch_pressure_bc(const StepArgs& a, cudaStream_t s);
// zeroGradient U / T patches take their owner cells' values (no-op without any)
void launch_zero_gradient_tu(const StepArgs& a, cudaStream_t s);
// Initial face values of mixed (rho fixedValue) patches; once, at creation.
void launch_ref_mixed_init(const StepArgs& a, const RefBuffers& b, cudaStream_t s);

// ------------------------------------------------------------- fused pipeline
struct FusedPlanDev;  // defined in fused_pipeline.cu

// -------------------------------------------------------------- common kernels
// g~,h~ <- gscale * Shakhov(rho,U,T,q=0) and tau <- tau(T,rho) for every cell.
template <typename S>
void launch_init_state(const StepArgs& a, S* gT, S* hT, double gscale, int sms, cudaStream_t s);
// Copy distributions between storage type S (scaled by gscale) and FP64 [nC][nV].
template <typename S>
void launch_export_dist(const StepArgs& a, const S* src, double* dst, double inv_gscale, int sms, cudaStream_t s);
template <typename S>
void launch_import_dist(const StepArgs& a, const double* src, S* dst, double gscale, int sms, cudaStream_t s);
// out[0] = max, out[1] = sum over internal faces of deltaCoeff*(|U_f| + sqrt(D) xi_max).
void launch_conum(const StepArgs& a, const double* dcI, double xi_max, double* out, cudaStream_t s);
// out = {sum|U-Uo|, sum|U|, sum|T-To|, sum T, sum|rho-rhoo|, sum rho}; then old <- current.
void launch_residual(const StepArgs& a, double* Uo, double* To, double* rhoo, double* out, cudaStream_t s);

}  // namespace dugks
