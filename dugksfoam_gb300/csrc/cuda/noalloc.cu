// Allocation-free cell macros: dugks_macros_noalloc.
//
// Some callers cannot allocate device memory at the point where they need
// the engine: code running inside another runtime that owns every device
// allocation (a memory pool or arena it hands out itself), or a solver loop
// that must not call cudaMalloc/cudaFree between time steps because those
// calls synchronise the device.  For them this file offers one entry point
// that allocates nothing: the macroscopic fields rho, U, T, q (updateMacroVol,
// fvDVM.C:597-728) of distributions the caller already holds on the device,
// written to output buffers the caller also provides.
//
// It is a variant of the cell-moment kernel (k_cell_mom in ref_pipeline.cu):
// the first kernel stores each cell's conserved moments (rho, rho U, rho E)
// in scratch, the second turns them into U and T and takes the heat-flux
// moment.  The scratch is the file-scope array below, sized for at most
// kNoAllocMaxCells cells (5 doubles each, 10 MiB); every GPU that loads the
// library holds it until the process exits.  All calls share it, so calls
// whose work overlaps on the GPU (two streams, two handles) race and must be
// serialised by the caller.  Each call overwrites every scratch entry it later
// reads, so nothing has to be cleared between calls.
//
// The array belongs to this file's device module: CUDA allocates it when it
// loads the module (at library load, or at the first call under lazy module
// loading), never inside a later call.  Its device address is looked up once
// per device, on the first call with that device current, and cached for the
// life of the process; a cudaDeviceReset ends the context that holds the
// array (and every handle's memory with it), so no call may follow a reset.
#include <cuda_runtime.h>

#include <mutex>

#include "device_common.cuh"
#include "dugks/dugks.h"
#include "kernels.h"
#include "noalloc.h"

namespace dugks {

static __device__ __align__(256) double g_noallocScratch[kNoAllocMaxCells * 5];

namespace {

// Device address of g_noallocScratch, looked up once per device (with that
// device current): in host code the symbol itself is only a stand-in.
constexpr int kMaxDevices = 64;
double* g_scratchAddr[kMaxDevices] = {};
std::mutex g_scratchMutex;

int scratch_address(int device, double** out, std::string& err) {
    if (device < 0 || device >= kMaxDevices) {
        err = "device ordinal out of range";
        return DUGKS_ERR_ARG;
    }
    std::lock_guard<std::mutex> lock(g_scratchMutex);
    if (!g_scratchAddr[device]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noallocScratch);
        if (e != cudaSuccess) {
            cudaGetLastError();
            err = std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e);
            return DUGKS_ERR_CUDA;
        }
        g_scratchAddr[device] = static_cast<double*>(p);
    }
    *out = g_scratchAddr[device];
    return DUGKS_OK;
}

constexpr int kThreads = 128;

// pass 1: conserved moments of every cell into scratch (DV order as P9)
__global__ void k_noalloc_conserved(StepArgs a, const double* __restrict__ g, const double* __restrict__ h,
                                    double* __restrict__ scratch) {
    __shared__ double red[32 * 5];
    const int c = blockIdx.x;
    const long long base = (long long)c * a.nV;
    double m[5] = {0, 0, 0, 0, 0};
    for (int v = threadIdx.x; v < a.nV; v += blockDim.x) {
        const double x0 = a.xi[v], x1 = a.xi[a.Vp + v], x2 = a.xi[2 * a.Vp + v], w = a.w[v];
        const double gv = g[base + v], hv = (a.hasH && h) ? h[base + v] : 0.0;
        m[0] += w * gv;
        m[1] += w * gv * x0;
        m[2] += w * gv * x1;
        m[3] += w * gv * x2;
        m[4] += 0.5 * w * ((x0 * x0 + x1 * x1 + x2 * x2) * gv + hv);
    }
    block_sum<5>(m, red);
    if (threadIdx.x == 0)
        for (int k = 0; k < 5; ++k) scratch[5 * (size_t)c + k] = m[k];
}

// pass 2: U, T, tau from the scratch moments, then the heat-flux moment
__global__ void k_noalloc_macros(StepArgs a, const double* __restrict__ g, const double* __restrict__ h,
                                 const double* __restrict__ scratch, double* rho, double* U, double* T, double* q) {
    __shared__ double red[32 * 3];
    const int c = blockIdx.x;
    const long long base = (long long)c * a.nV;
    const double r = scratch[5 * (size_t)c];
    const double Ux = scratch[5 * (size_t)c + 1] / r, Uy = scratch[5 * (size_t)c + 2] / r,
                 Uz = scratch[5 * (size_t)c + 3] / r;
    const double Tc = (scratch[5 * (size_t)c + 4] - 0.5 * r * (Ux * Ux + Uy * Uy + Uz * Uz)) / ((a.K + 3) / 2.0 * a.R * r);
    const double tau = tau_ref(Tc, r, a.muRef, a.omega, a.Tref, a.R);
    double qq[3] = {0, 0, 0};
    for (int v = threadIdx.x; v < a.nV; v += blockDim.x) {
        const double x0 = a.xi[v], x1 = a.xi[a.Vp + v], x2 = a.xi[2 * a.Vp + v], w = a.w[v];
        const double gv = g[base + v], hv = (a.hasH && h) ? h[base + v] : 0.0;
        const double c0 = x0 - Ux, c1 = x1 - Uy, c2 = x2 - Uz;
        const double s = (c0 * c0 + c1 * c1 + c2 * c2) * gv + hv;
        qq[0] += 0.5 * w * c0 * s;
        qq[1] += 0.5 * w * c1 * s;
        qq[2] += 0.5 * w * c2 * s;
    }
    block_sum<3>(qq, red);
    if (threadIdx.x == 0) {
        const double fac = 2.0 * tau / (2.0 * tau + a.dt * a.Pr);
        if (rho) rho[c] = r;
        if (U) { U[3 * c] = Ux; U[3 * c + 1] = Uy; U[3 * c + 2] = Uz; }
        if (T) T[c] = Tc;
        if (q) { q[3 * c] = fac * qq[0]; q[3 * c + 1] = fac * qq[1]; q[3 * c + 2] = fac * qq[2]; }
    }
}

}  // namespace

int macros_noalloc(const StepArgs& a, int device, cudaStream_t s, const double* g, const double* h, double* rho,
                   double* U, double* T, double* q, std::string& err) {
    if (!g || (a.hasH && !h)) {
        err = "dugks_macros_noalloc: missing input distribution";
        return DUGKS_ERR_ARG;
    }
    if (a.nC > kNoAllocMaxCells) {
        err = "dugks_macros_noalloc: " + std::to_string(a.nC) + " cells exceed the scratch limit of " +
              std::to_string(kNoAllocMaxCells) + " cells";
        return DUGKS_ERR_ARG;
    }
    if (a.nC == 0) return DUGKS_OK;
    {  // an error left by the caller's earlier work is not this call's: report it, launch nothing
        const cudaError_t pending = cudaPeekAtLastError();
        if (pending != cudaSuccess) {
            err = std::string("dugks_macros_noalloc: CUDA error pending before the call: ") +
                  cudaGetErrorString(pending);
            return DUGKS_ERR_CUDA;
        }
    }
    double* scratch = nullptr;
    if (int e = scratch_address(device, &scratch, err)) return e;
    k_noalloc_conserved<<<a.nC, kThreads, 0, s>>>(a, g, h, scratch);
    k_noalloc_macros<<<a.nC, kThreads, 0, s>>>(a, g, h, scratch, rho, U, T, q);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        err = std::string("dugks_macros_noalloc launch: ") + cudaGetErrorString(e);
        return DUGKS_ERR_CUDA;
    }
    return DUGKS_OK;
}

}  // namespace dugks
