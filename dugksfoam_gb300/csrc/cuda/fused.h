// Fused tile-sweep pipeline interface (implementation: fused_pipeline.cu).
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
    virtual void exportDist(const StepArgs& a, int which, double* dst, int sms, cudaStream_t s) = 0;
    virtual void importDist(const StepArgs& a, int which, const double* src, int sms, cudaStream_t s) = 0;
    virtual void* distPtr(int which) = 0;   // current g~ (0) / h~ (1)
    virtual void* gradBPtr(int which) = 0;  // current lagged boundary gradient
};

std::unique_ptr<FusedPipeline> make_fused_pipeline(Solver& s, const StepArgs& a, int precision, std::string& err);

}  // namespace dugks
