// Fused tile-sweep pipeline interface (implementation: fused_pipeline_impl.cuh).
#pragma once

#include <cuda_runtime.h>

#include <memory>
#include <string>

#include "device_common.cuh"

namespace dugks {

class Solver;

class FusedPipeline {
public:
    virtual ~FusedPipeline() = default;
    // Density scale of the stored distributions (stored = gscale * physical).
    virtual double gscale() const = 0;
    virtual void initState(const StepArgs& a, int sms, cudaStream_t s) = 0;
    virtual int nKernels() const = 0;
    virtual const char* kernelName(int k) const = 0;
    virtual void launch(int k, const StepArgs& a, int sms, cudaStream_t s) = 0;
    // After the launches of one step: swap double buffers (cell macros in base).
    virtual void endStep(StepArgs& base) = 0;
    // Recompute state derived from the cell macros (after a checkpoint load).
    virtual void refreshDerived(const StepArgs& a, int sms, cudaStream_t s) = 0;
    virtual void exportDist(const StepArgs& a, int which, double* dst, int sms, cudaStream_t s) = 0;
    virtual void importDist(const StepArgs& a, int which, const double* src, int sms, cudaStream_t s) = 0;
    virtual void* distPtr(int which) = 0;   // current g~ (0) / h~ (1)
    virtual void* gradBPtr(int which) = 0;  // current lagged boundary gradient
    virtual size_t bytes() const = 0;
    virtual std::string describe() const = 0;
};

// DVs per lane of the fused kernels for a precision (FP32: DUGKS_NPL, default 4).
int fused_npl(int precision);
// DV chunk granularity the fused kernels need (the padded DV count must be a multiple).
int fused_dv_granule(int precision);

std::unique_ptr<FusedPipeline> make_fused_pipeline(Solver& s, const StepArgs& a, int precision, std::string& err);
std::unique_ptr<FusedPipeline> make_fused_fp32(Solver& s, const StepArgs& a, std::string& err);
std::unique_ptr<FusedPipeline> make_fused_fp64(Solver& s, const StepArgs& a, std::string& err);

}  // namespace dugks
