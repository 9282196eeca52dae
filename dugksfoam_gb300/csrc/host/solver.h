// dugks::Solver -- host-side owner of one DUGKS case on one GPU.
//
// Mirrors the reference's Foam::fvDVM (src/fvDVM/fvDVM/fvDVM.H:78-377):
// evolution(), getCoNum(), rhoVol()/Uvol()/Tvol()/qVol()/tauVol(), with the
// state resident in device memory and the step run as CUDA kernels.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <memory>
#include <string>
#include <vector>

#include "../cuda/kernels.h"
#include "dugks/dugks.h"
#include "mesh.h"

namespace dugks {

class FusedPipeline;  // fused_pipeline.cu

class Solver {
public:
    static std::unique_ptr<Solver> create(const dugks_case_desc& d, std::string& err, int& code);
    ~Solver();

    // fvDVM::evolution() n times (asynchronous)
    int evolution(int n);
    int synchronize();
    int getCoNum(double& maxCo, double& meanCo);
    int macros(double* rho, double* U, double* T, double* q, double* tau);
    int faceMacros(double* rho, double* U, double* T, double* q, double* tau);
    int wall(int patch, double* rhoW, double* qWall, double* stressWall);
    // rho, U, T patch values of a non-empty patch (rho: Maxwell-wall density on walls)
    int boundary(int patch, double* rho, double* U, double* T);
    int residual(double res[3]);
    int getDist(double* g, double* h);
    int setDist(const double* g, const double* h);
    size_t checkpointSize() const;
    int checkpointSave(void* buf, size_t n);
    int checkpointLoad(const void* buf, size_t n);
    int profile(int nsteps, std::vector<std::string>& names, std::vector<double>& ms);
    int launchesPerStep() const;
    void info(dugks_info& out) const;

    void setDt(double dt) { dt_ = dt; }
    double dt() const { return dt_; }
    int setStream(cudaStream_t s);
    cudaStream_t stream() const { return stream_; }
    const std::string& error() const { return err_; }
    const Mesh& mesh() const { return mesh_; }
    // Step arguments with the current dt (device pointers of the handle).
    StepArgs stepArgs() const { return argsNow(); }
    int device() const { return device_; }
    int sms() const { return sms_; }
    // batched stepping: the FP32 pipeline, and the bookkeeping of n steps that
    // ran outside evolution() (double-buffer swaps, step count)
    FusedPipeline* fusedPipeline() const { return fused_.get(); }
    void advanceExternal(int n);
    // initial fields rho0, U0, T0 on the device (the state dugks_create starts from)
    const double* initRho() const { return initRho_; }
    const double* initU() const { return initU_; }
    const double* initT() const { return initT_; }

    // internal: allocation helper (recorded for release)
    template <typename T>
    T* dalloc(size_t n);
    int fail(int code, const std::string& msg);
    int checkCuda(cudaError_t e, const char* what);
    // Wait for the stream and report the status word the kernels set, in one
    // host round trip (the word is copied into pinned memory behind the work).
    int syncStatus(const char* what);

private:
    Solver() = default;
    int init(const dugks_case_desc& d);
    int runStep(bool timed, std::vector<double>* ms, std::vector<cudaEvent_t>* ev);
    StepArgs argsNow() const;

    Mesh mesh_;
    std::string err_;
    int device_ = 0, sms_ = 132;
    int precision_ = DUGKS_FP64, pipeline_ = DUGKS_PIPE_REFERENCE;
    int nV_ = 0, Vp_ = 0, hasH_ = 1, nXiPerDim_ = 0;
    double dt_ = 0.0, xiMax_ = 0.0, gscale_ = 1.0;
    int64_t steps_ = 0;
    cudaStream_t ownStream_ = nullptr, stream_ = nullptr;
    std::vector<void*> allocs_;
    size_t bytes_ = 0;
    bool oom_ = false;
    StepArgs base_{};
    // mesh-side device arrays not in StepArgs
    double* dcI_ = nullptr;
    double *initRho_ = nullptr, *initU_ = nullptr, *initT_ = nullptr;
    // reference pipeline buffers (FP64)
    RefBuffers ref_{};
    // residual "old" fields and scratch
    double *Uo_ = nullptr, *To_ = nullptr, *ro_ = nullptr, *red_ = nullptr;
    // pinned host words: [0] the status word, [8..] reduction results (doubles)
    unsigned char* pin_ = nullptr;
    int* pinStatus() const { return reinterpret_cast<int*>(pin_); }
    double* pinRed() const { return reinterpret_cast<double*>(pin_ + 8); }
    // fused pipeline
    std::unique_ptr<FusedPipeline> fused_;
    std::vector<int32_t> patchFirstWall_, patchNWall_;
};

}  // namespace dugks
