// Fused sweeps with FP32 distributions (FP64 moments and macros).
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

bool fused_batch_prepare(BatchLaunch& L, int sms) {
    return dispatch2d(L, [&](auto K) { return decltype(K)::prepare(L, sms); });
}

void fused_batch_launch(int k, const BatchLaunch& L, int sms, cudaStream_t s) {
    dispatch2d(L, [&](auto K) {
        decltype(K)::launch(k, L, sms, s);
        return true;
    });
}

}  // namespace dugks
