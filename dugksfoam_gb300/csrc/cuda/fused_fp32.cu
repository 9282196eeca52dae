// Fused sweeps with FP32 distributions (FP64 moments and macros).
#include <algorithm>

#include "fused_pipeline_impl.cuh"

namespace dugks {

std::unique_ptr<FusedPipeline> make_fused_fp32(Solver& s, const StepArgs& a, std::string& err) {
    std::unique_ptr<FusedPipelineT<float>> p(new FusedPipelineT<float>());
    if (!p->init(s, a, err)) return nullptr;
    return p;
}

}  // namespace dugks

namespace dugks {
namespace {

constexpr int kBatchWarps = 16;   // face sides: warps per tile block
constexpr int kBatchGather = 8;   // cell gather: warps per block

template <int D, bool H, int NPL>
struct BatchKernels {
    static bool prepare(BatchLaunch& L, int sms) {
        auto kf = k_face_sides32_batch<D, H, NPL, kBatchWarps>;
        auto kg = k_cell_gather32_batch<D, H, NPL, kBatchGather>;
        if (allow_max_dynamic_smem(kf) != cudaSuccess || allow_max_dynamic_smem(kg) != cudaSuccess) {
            cudaGetLastError();
            return false;
        }
        int per = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kg, kBatchGather * 32, L.gatherSmem);
        L.gatherBlocks = std::max(1, per) * std::max(1, sms);
        return true;
    }
    static bool persistentPrepare(BatchLaunch& L, int sms) {
        auto kp = k_batch_persistent32<D, H, NPL, kBatchWarps>;
        const size_t gsm = persist_gather_smem<D, H>(kBatchWarps, L.MF, 32 * NPL);
        L.persistSmem = std::max(L.smemFace, gsm);
        int dev = 0, maxSmem = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&maxSmem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
        cudaFuncAttributes fa{};
        if (cudaFuncGetAttributes(&fa, kp) != cudaSuccess) { cudaGetLastError(); return false; }
        if (L.persistSmem + fa.sharedSizeBytes > (size_t)maxSmem) return false;
        if (allow_max_dynamic_smem(kp) != cudaSuccess) { cudaGetLastError(); return false; }
        int per = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kp, kBatchWarps * 32, L.persistSmem) != cudaSuccess ||
            per < 1) {
            cudaGetLastError();
            return false;
        }
        L.persistBlocks = per * std::max(1, sms);  // every block resident: the grid barriers need it
        return true;
    }
    static cudaError_t persistentLaunch(const BatchLaunch& L0, const BatchLaunch& L1, int nSteps, int parity0,
                                        unsigned* bar, long long cap, int* status, cudaStream_t s) {
        const FusedArgs<float>* A0 = static_cast<const FusedArgs<float>*>(L0.args);
        const FusedArgs<float>* A1 = static_cast<const FusedArgs<float>*>(L1.args);
        const int2* work = L0.work;
        int nWork = L0.nWork, nCases = L0.nCases, MF = L0.MF;
        const int* fo = L0.faceOff;
        const int* co = L0.cellOff;
        void* args[] = {&A0, &A1, &work, &nWork, &fo, &co, &nCases, &MF, &nSteps, &parity0, &bar, &cap, &status};
        return cudaLaunchCooperativeKernel(reinterpret_cast<const void*>(k_batch_persistent32<D, H, NPL, kBatchWarps>),
                                           dim3(L0.persistBlocks), dim3(kBatchWarps * 32), args, L0.persistSmem, s);
    }
    static void launch(int k, const BatchLaunch& L, int sms, cudaStream_t s) {
        const FusedArgs<float>* AA = static_cast<const FusedArgs<float>*>(L.args);
        if (k == 0)
            k_face_sides32_batch<D, H, NPL, kBatchWarps><<<L.nWork, kBatchWarps * 32, L.smemFace, s>>>(AA, L.work);
        else if (k == 1)  // one face per thread: FP64-bound, wants every warp it can get
            k_face_macros32_batch<D, H><<<std::max(1, (L.nFaces + 127) / 128), 128, 0, s>>>(AA, L.faceOff, L.nCases);
        else
            k_cell_gather32_batch<D, H, NPL, kBatchGather><<<L.gatherBlocks, kBatchGather * 32, L.gatherSmem, s>>>(
                AA, L.cellOff, L.nCases, L.MF);
    }
};

template <typename F>
bool dispatch2d(const BatchLaunch& L, F&& f) {
    if (L.D != 2) return false;
    if (L.H && L.npl == 4) return f(BatchKernels<2, true, 4>());
    if (L.H && L.npl == 2) return f(BatchKernels<2, true, 2>());
    if (!L.H && L.npl == 4) return f(BatchKernels<2, false, 4>());
    if (!L.H && L.npl == 2) return f(BatchKernels<2, false, 2>());
    return false;
}

}  // namespace

size_t fused_gather_smem(int nw, int mf, int kc, bool h) { return gather_smem(nw, mf, kc, h); }

bool fused_batch_prepare(BatchLaunch& L, int sms) {
    return dispatch2d(L, [&](auto K) { return decltype(K)::prepare(L, sms); });
}

bool fused_batch_persistent_prepare(BatchLaunch& L, int sms) {
    return dispatch2d(L, [&](auto K) { return decltype(K)::persistentPrepare(L, sms); });
}

cudaError_t fused_batch_persistent_launch(const BatchLaunch& L0, const BatchLaunch& L1, int nSteps, int parity0,
                                          unsigned* bar, long long cap, int* status, cudaStream_t s) {
    cudaError_t r = cudaErrorInvalidConfiguration;
    dispatch2d(L0, [&](auto K) {
        r = decltype(K)::persistentLaunch(L0, L1, nSteps, parity0, bar, cap, status, s);
        return true;
    });
    return r;
}

void fused_batch_launch(int k, const BatchLaunch& L, int sms, cudaStream_t s) {
    dispatch2d(L, [&](auto K) {
        decltype(K)::launch(k, L, sms, s);
        return true;
    });
}

}  // namespace dugks
