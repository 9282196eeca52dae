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

    // ---- batched stepping of several cases (FP32 pipeline only)
    virtual bool batchable() const { return false; }        // may join a batch (FP32 pipeline)
    virtual bool batchKernels() const { return false; }     // fits the batched kernels (diffuse walls only)
    // Kernel arguments (a FusedArgs<float>) of the step that starts `parity`
    // steps from now (0 or 1), for base arguments `a` of the current step.
    virtual void batchArgs(const StepArgs& a, int parity, void* out) const { (void)a; (void)parity; (void)out; }
    virtual size_t batchArgsBytes() const { return 0; }
    virtual int batchTiles() const { return 0; }
    virtual size_t batchSmemFace() const { return 0; }
    virtual int batchGatherMF() const { return 0; }
    virtual int batchNpl() const { return 0; }
    // Launch the step `parity` steps ahead (kernels only: no host bookkeeping),
    // e.g. into a graph capture.
    virtual void launchParity(const StepArgs& a, int parity, int sms, cudaStream_t s) {
        (void)a; (void)parity; (void)sms; (void)s;
    }
};

// One launch over several cases: kernel k (0 face sides, 1 face macros,
// 2 cell gather) of the FP32 step for every case.
struct BatchLaunch {
    const void* args = nullptr;  // device FusedArgs<float>[nCases] of this step
    const int2* work = nullptr;  // [nWork] (case, tile)
    int nWork = 0;
    const int* faceOff = nullptr;  // [nCases+1] first global active face of each case
    const int* cellOff = nullptr;  // [nCases+1] first global cell of each case
    int nCases = 0;
    int nFaces = 0;  // active faces of all cases
    size_t smemFace = 0;
    int MF = 0;
    size_t gatherSmem = 0;
    int gatherBlocks = 1;
    int D = 2, H = 1, npl = 4;
    // persistent kernel (all passes and steps in one cooperative launch)
    size_t persistSmem = 0;
    int persistBlocks = 0;
};
// Set function attributes and the persistent gather grid; false if the
// (D, H, npl) combination has no kernels.
bool fused_batch_prepare(BatchLaunch& L, int sms);
// Dynamic shared memory of the FP32 gather sweep for nw warps per block, MF
// staged faces per cell and a DV chunk of kc velocities (with h or not).
size_t fused_gather_smem(int nw, int mf, int kc, bool h);
void fused_batch_launch(int k, const BatchLaunch& L, int sms, cudaStream_t s);
// The persistent batched kernel: shared memory and the co-resident grid
// (false if it does not fit), and one cooperative launch of nSteps steps from
// parity0 (L0 / L1: the launch descriptions of parity 0 / 1).  bar: two
// zeroed unsigned counters; status receives DUGKS_ERR_TIMEOUT when a grid
// barrier wait gives up after cap polls.
bool fused_batch_persistent_prepare(BatchLaunch& L, int sms);
cudaError_t fused_batch_persistent_launch(const BatchLaunch& L0, const BatchLaunch& L1, int nSteps, int parity0,
                                          unsigned* bar, long long cap, int* status, cudaStream_t s);

// Allow a kernel the device's opt-in maximum of dynamic shared memory (less
// its static shared memory).  The limit belongs to the kernel function, which
// every case launching it shares, so it is set once to the maximum and each
// launch asks for its own size.
template <typename F>
inline cudaError_t allow_max_dynamic_smem(F* func) {
    int dev = 0, maxSmem = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&maxSmem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    cudaFuncAttributes fa{};
    if (cudaError_t e = cudaFuncGetAttributes(&fa, reinterpret_cast<const void*>(func))) return e;
    return cudaFuncSetAttribute(reinterpret_cast<const void*>(func), cudaFuncAttributeMaxDynamicSharedMemorySize,
                                maxSmem - (int)fa.sharedSizeBytes);
}

// Tuning override for pipelines created while it is set (0 = default):
// DVs per lane and the tile-size cap of the face sweep.
// waveBalance: size the FP32 face-sweep tiles to fill whole waves of the SMs
// (a case whose tiles share the grid with other cases' passes false)
void fused_set_tuning(int npl, int maxTileCells, bool waveBalance = true);
int fused_tile_cap();
bool fused_wave_balance();

// DVs per lane of the fused kernels for a precision (FP32: DUGKS_NPL, default 4).
int fused_npl(int precision);
// FP32 face sweep with per-cell gradients also in 2D (DUGKS_FACE_GRAD=1; 3D always).
bool fused_face_grad();
// DV chunk granularity the fused kernels need (the padded DV count must be a multiple).
int fused_dv_granule(int precision);

std::unique_ptr<FusedPipeline> make_fused_pipeline(Solver& s, const StepArgs& a, int precision, std::string& err);
std::unique_ptr<FusedPipeline> make_fused_fp32(Solver& s, const StepArgs& a, std::string& err);
std::unique_ptr<FusedPipeline> make_fused_fp64(Solver& s, const StepArgs& a, std::string& err);

}  // namespace dugks
