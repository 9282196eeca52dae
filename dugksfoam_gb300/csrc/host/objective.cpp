// Gradient harness of the FP64 step: objective value, tangent-linear
// directional derivative and adjoint gradient with respect to the wall
// temperatures and the viscosity scale (see gradient.h).
#include "objective.h"

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "../cuda/gradient.h"
#include "../cuda/kernels.h"

namespace dugks {
namespace {

class Work {
public:
    explicit Work(Solver& s) : s_(s) {}
    ~Work() {
        for (void* p : allocs_) cudaFree(p);
    }
    template <typename T>
    T* alloc(size_t n) {
        void* p = nullptr;
        if (cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T)) != cudaSuccess) {
            cudaGetLastError();
            oom = true;
            return nullptr;
        }
        cudaMemsetAsync(p, 0, std::max<size_t>(n, 1) * sizeof(T), s_.stream());
        allocs_.push_back(p);
        return static_cast<T*>(p);
    }
    bool oom = false;

private:
    Solver& s_;
    std::vector<void*> allocs_;
};

// FP64 reference-pipeline forward on private buffers and macros.
struct Fwd {
    StepArgs a{};
    RefBuffers b{};
};

bool make_fwd(Solver& s, Work& W, Fwd& f) {
    f.a = s.stepArgs();
    StepArgs& a = f.a;
    const size_t nC = a.nC, nA = a.nA, nW = std::max(a.nW, 1), Vp = a.Vp, D = a.D;
    a.rho = W.alloc<double>(nC); a.U = W.alloc<double>(3 * nC); a.T = W.alloc<double>(nC);
    a.q = W.alloc<double>(3 * nC); a.tau = W.alloc<double>(nC);
    a.rhoF = W.alloc<double>(nA); a.UF = W.alloc<double>(3 * nA); a.TF = W.alloc<double>(nA);
    a.qF = W.alloc<double>(3 * nA); a.tauF = W.alloc<double>(nA);
    a.rhoW = W.alloc<double>(nW); a.qWall = W.alloc<double>(3 * nW); a.stressWall = W.alloc<double>(9 * nW);
    a.status = W.alloc<int>(1);
    RefBuffers& b = f.b;
    b.gT = W.alloc<double>(nC * Vp); b.gB = W.alloc<double>(nC * Vp); b.gG = W.alloc<double>(nC * D * Vp);
    b.Gbg = W.alloc<double>(nW * Vp); b.gS = W.alloc<double>(nA * Vp);
    if (a.hasH) {
        b.hT = W.alloc<double>(nC * Vp); b.hB = W.alloc<double>(nC * Vp); b.hG = W.alloc<double>(nC * D * Vp);
        b.Gbh = W.alloc<double>(nW * Vp); b.hS = W.alloc<double>(nA * Vp);
    }
    return !W.oom;
}

void fwd_init(Solver& s, Fwd& f) {
    StepArgs& a = f.a;
    cudaStream_t st = s.stream();
    const size_t nC = a.nC;
    cudaMemcpyAsync(a.rho, s.initRho(), nC * 8, cudaMemcpyDeviceToDevice, st);
    cudaMemcpyAsync(a.U, s.initU(), 3 * nC * 8, cudaMemcpyDeviceToDevice, st);
    cudaMemcpyAsync(a.T, s.initT(), nC * 8, cudaMemcpyDeviceToDevice, st);
    cudaMemsetAsync(a.q, 0, 3 * nC * 8, st);
    cudaMemsetAsync(f.b.Gbg, 0, (size_t)std::max(a.nW, 1) * a.Vp * 8, st);
    if (a.hasH) cudaMemsetAsync(f.b.Gbh, 0, (size_t)std::max(a.nW, 1) * a.Vp * 8, st);
    launch_init_state<double>(a, f.b.gT, f.b.hT, 1.0, s.sms(), st);  // Shakhov(rho0, U0, T0, 0); tau0
}

bool in_window(const Objective& o, int n) { return n >= o.avgFirst && n < o.nSteps; }
double window_scale(const Objective& o) { return 1.0 / std::max(1, o.nSteps - o.avgFirst); }

void fwd_step(Solver& s, Fwd& f, const Objective& o, int n, const double* wq, const double* ws, double* J,
              int lastPass = kRefKernels - 1, int firstPass = 0) {
    for (int k = firstPass; k <= lastPass; ++k) {
        launch_ref_pass(k, f.a, f.b, s.sms(), s.stream());
        if (k == 4 && J && in_window(o, n)) launch_objective(f.a, wq, ws, window_scale(o), J, s.stream());
    }
}

// Objective weights per wall face: S_w on the heat-flux patch, |S_w| on the
// shear patch.
int weights(Solver& s, const Objective& o, Work& W, double*& wq, double*& ws) {
    const Mesh& m = s.mesh();
    const int nW = m.nW;
    std::vector<double> hq(3 * (size_t)std::max(nW, 1), 0.0), hs(std::max(nW, 1), 0.0);
    for (int w = 0; w < nW; ++w) {
        const double* S = &m.Sf[3 * (size_t)m.wallFace[w]];
        if (m.wallPatch[w] == o.qPatch)
            for (int k = 0; k < 3; ++k) hq[3 * w + k] = S[k];
        if (m.wallPatch[w] == o.stressPatch) hs[w] = std::sqrt(S[0] * S[0] + S[1] * S[1] + S[2] * S[2]);
    }
    wq = W.alloc<double>(hq.size());
    ws = W.alloc<double>(hs.size());
    if (W.oom) return s.fail(DUGKS_ERR_OOM, "gradient: device allocation failed");
    cudaMemcpyAsync(wq, hq.data(), hq.size() * 8, cudaMemcpyHostToDevice, s.stream());
    cudaMemcpyAsync(ws, hs.data(), hs.size() * 8, cudaMemcpyHostToDevice, s.stream());
    return DUGKS_OK;
}

int check(Solver& s, const Objective& o) {
    if (o.nSteps < 1 || o.avgFirst < 0 || o.avgFirst >= o.nSteps)
        return s.fail(DUGKS_ERR_ARG, "objective: need 0 <= avg_first < n_steps");
    if (o.ckptEvery < 1) return s.fail(DUGKS_ERR_ARG, "objective: checkpoint_every must be >= 1");
    if (!(s.dt() > 0)) return s.fail(DUGKS_ERR_ARG, "objective: set dt first");
    for (int32_t k : s.mesh().wallKind)
        if (k != DUGKS_PATCH_MAXWELL)
            return s.fail(DUGKS_ERR_UNSUPPORTED, "objective: the differentiated step takes diffuse walls only");
    return s.synchronize();
}

int finish(Solver& s, const char* what) {
    cudaError_t ce = cudaStreamSynchronize(s.stream());
    if (ce == cudaSuccess) ce = cudaGetLastError();
    return s.checkCuda(ce, what);
}

}  // namespace

int objective_value(Solver& s, const Objective& o, double& J) {
    if (int e = check(s, o)) return e;
    Work W(s);
    Fwd f;
    double *wq, *ws;
    if (!make_fwd(s, W, f)) return s.fail(DUGKS_ERR_OOM, "objective: device allocation failed");
    if (int e = weights(s, o, W, wq, ws)) return e;
    double* dJ = W.alloc<double>(1);
    fwd_init(s, f);
    for (int n = 0; n < o.nSteps; ++n) fwd_step(s, f, o, n, wq, ws, dJ);
    cudaMemcpyAsync(&J, dJ, 8, cudaMemcpyDeviceToHost, s.stream());
    return finish(s, "objective value");
}

int objective_tangent(Solver& s, const Objective& o, const double* dTw, double dMuScale, double& J, double& dJ) {
    if (int e = check(s, o)) return e;
    Work W(s);
    double *wq, *ws;
    if (int e = weights(s, o, W, wq, ws)) return e;
    TlmState t{};
    t.a = s.stepArgs();
    const StepArgs& a = t.a;
    const size_t nC = a.nC, nA = a.nA, nW = std::max(a.nW, 1), Vp = a.Vp, D = a.D;
    t.gT = W.alloc<Dual>(nC * Vp); t.gB = W.alloc<Dual>(nC * Vp); t.gG = W.alloc<Dual>(nC * D * Vp);
    t.Gbg = W.alloc<Dual>(nW * Vp); t.gS = W.alloc<Dual>(nA * Vp);
    if (a.hasH) {
        t.hT = W.alloc<Dual>(nC * Vp); t.hB = W.alloc<Dual>(nC * Vp); t.hG = W.alloc<Dual>(nC * D * Vp);
        t.Gbh = W.alloc<Dual>(nW * Vp); t.hS = W.alloc<Dual>(nA * Vp);
    }
    t.rho = W.alloc<Dual>(nC); t.U = W.alloc<Dual>(3 * nC); t.T = W.alloc<Dual>(nC); t.q = W.alloc<Dual>(3 * nC);
    t.tau = W.alloc<Dual>(nC);
    t.rhoF = W.alloc<Dual>(nA); t.UF = W.alloc<Dual>(3 * nA); t.TF = W.alloc<Dual>(nA); t.qF = W.alloc<Dual>(3 * nA);
    t.tauF = W.alloc<Dual>(nA);
    t.rhoW = W.alloc<Dual>(nW); t.qWall = W.alloc<Dual>(3 * nW); t.stressWall = W.alloc<Dual>(9 * nW);
    t.Tw = W.alloc<Dual>(nW); t.incAbs = W.alloc<Dual>(nW);
    t.a.status = W.alloc<int>(1);
    Dual* dJd = W.alloc<Dual>(1);
    if (W.oom) return s.fail(DUGKS_ERR_OOM, "tangent: device allocation failed");
    std::vector<double> tw(nW, 0.0);
    if (a.nW) cudaMemcpy(tw.data(), a.Tw, a.nW * 8, cudaMemcpyDeviceToHost);
    std::vector<Dual> twd(nW);
    for (int w = 0; w < a.nW; ++w) twd[w] = Dual{tw[w], dTw ? dTw[w] : 0.0};
    cudaMemcpyAsync(t.Tw, twd.data(), nW * sizeof(Dual), cudaMemcpyHostToDevice, s.stream());
    t.muRef = Dual{a.muRef, a.muRef * dMuScale};
    if (a.nW) tlm_launch_incabs(t, s.stream());
    tlm_launch_init(t, s.initRho(), s.initU(), s.initT(), s.sms(), s.stream());
    for (int n = 0; n < o.nSteps; ++n)
        tlm_launch_step(t, in_window(o, n), wq, ws, window_scale(o), dJd, s.sms(), s.stream());
    Dual r{};
    cudaMemcpyAsync(&r, dJd, sizeof(Dual), cudaMemcpyDeviceToHost, s.stream());
    if (int e = finish(s, "tangent")) return e;
    J = r.v;
    dJ = r.d;
    return DUGKS_OK;
}

int objective_adjoint(Solver& s, const Objective& o, double& J, double* dJdTw, double& dJdMuScale) {
    if (int e = check(s, o)) return e;
    Work W(s);
    Fwd f;
    double *wq, *ws;
    if (!make_fwd(s, W, f)) return s.fail(DUGKS_ERR_OOM, "adjoint: device allocation failed");
    if (int e = weights(s, o, W, wq, ws)) return e;
    const StepArgs& a = f.a;
    cudaStream_t st = s.stream();
    const int sms = s.sms();
    const size_t nC = a.nC, nA = a.nA, nW = std::max(a.nW, 1), Vp = a.Vp, D = a.D, H = a.hasH ? 2 : 1;
    // one stored state: g~ (, h~), G_b (g, h), cell macros rho U T q tau
    const size_t oG = 0, oH = nC * Vp, oBg = H * nC * Vp, oBh = oBg + nW * Vp, oM = oBg + H * nW * Vp;
    const size_t stateN = oM + 9 * nC;
    auto save = [&](double* dst) {
        cudaMemcpyAsync(dst + oG, f.b.gT, nC * Vp * 8, cudaMemcpyDeviceToDevice, st);
        if (a.hasH) cudaMemcpyAsync(dst + oH, f.b.hT, nC * Vp * 8, cudaMemcpyDeviceToDevice, st);
        cudaMemcpyAsync(dst + oBg, f.b.Gbg, nW * Vp * 8, cudaMemcpyDeviceToDevice, st);
        if (a.hasH) cudaMemcpyAsync(dst + oBh, f.b.Gbh, nW * Vp * 8, cudaMemcpyDeviceToDevice, st);
        double* m = dst + oM;
        cudaMemcpyAsync(m, a.rho, nC * 8, cudaMemcpyDeviceToDevice, st);
        cudaMemcpyAsync(m + nC, a.U, 3 * nC * 8, cudaMemcpyDeviceToDevice, st);
        cudaMemcpyAsync(m + 4 * nC, a.T, nC * 8, cudaMemcpyDeviceToDevice, st);
        cudaMemcpyAsync(m + 5 * nC, a.q, 3 * nC * 8, cudaMemcpyDeviceToDevice, st);
        cudaMemcpyAsync(m + 8 * nC, a.tau, nC * 8, cudaMemcpyDeviceToDevice, st);
    };
    auto restore = [&](const double* src) {
        cudaMemcpyAsync(f.b.gT, src + oG, nC * Vp * 8, cudaMemcpyDeviceToDevice, st);
        if (a.hasH) cudaMemcpyAsync(f.b.hT, src + oH, nC * Vp * 8, cudaMemcpyDeviceToDevice, st);
        cudaMemcpyAsync(f.b.Gbg, src + oBg, nW * Vp * 8, cudaMemcpyDeviceToDevice, st);
        if (a.hasH) cudaMemcpyAsync(f.b.Gbh, src + oBh, nW * Vp * 8, cudaMemcpyDeviceToDevice, st);
        const double* m = src + oM;
        cudaMemcpyAsync(a.rho, m, nC * 8, cudaMemcpyDeviceToDevice, st);
        cudaMemcpyAsync(a.U, m + nC, 3 * nC * 8, cudaMemcpyDeviceToDevice, st);
        cudaMemcpyAsync(a.T, m + 4 * nC, nC * 8, cudaMemcpyDeviceToDevice, st);
        cudaMemcpyAsync(a.q, m + 5 * nC, 3 * nC * 8, cudaMemcpyDeviceToDevice, st);
        cudaMemcpyAsync(a.tau, m + 8 * nC, nC * 8, cudaMemcpyDeviceToDevice, st);
    };
    // the reverse kernels tabulate the Maxwellian per direction of the tensor-product grid
    int M = 1;
    while ((D == 3 ? (size_t)M * M * M : (size_t)M * M) < (size_t)a.nV) ++M;
    if ((D != 2 && D != 3) || (D == 3 ? M * M * M : M * M) != a.nV || adj_table_bytes(a.D, M) > 48 * 1024)
        return s.fail(DUGKS_ERR_UNSUPPORTED, "adjoint: needs a 2D or 3D tensor-product velocity grid of at most 512 "
                                             "points per direction");
    const int K = o.ckptEvery, N = o.nSteps, nSeg = (N + K - 1) / K;
    double* ckpt = W.alloc<double>(stateN * (size_t)nSeg);
    double* seg = W.alloc<double>(stateN * (size_t)(K + 1));
    // Per-step forward values the reverse reads (face values before relaxation,
    // face macros, rho_w), kept for a whole segment when device memory allows;
    // otherwise each reverse step recomputes P1..P6 from its stored state.
    const size_t iS = 0, iSh = nA * Vp, iF = H * nA * Vp, iW = iF + 9 * nA, interN = iW + nW;
    double* inter = nullptr;
    {
        size_t freeB = 0, totalB = 0;
        cudaMemGetInfo(&freeB, &totalB);
        const char* rc = std::getenv("DUGKS_ADJ_RECOMPUTE");  // force the recompute form
        if (!(rc && rc[0] == '1') && interN * (size_t)K * 8 < freeB / 2) inter = W.alloc<double>(interN * (size_t)K);
        if (W.oom) { cudaGetLastError(); W.oom = false; inter = nullptr; }
    }
    double* dJ = W.alloc<double>(1);
    // adjoint buffers
    AdjState A{};
    A.lgN = W.alloc<double>(nC * Vp); A.lgT = W.alloc<double>(nC * Vp); A.lgB = W.alloc<double>(nC * Vp);
    A.lG = W.alloc<double>(nC * D * Vp); A.lgS = W.alloc<double>(nA * Vp);
    A.lGbN = W.alloc<double>(nW * Vp); A.lGb = W.alloc<double>(nW * Vp);
    if (a.hasH) {
        A.lhN = W.alloc<double>(nC * Vp); A.lhT = W.alloc<double>(nC * Vp); A.lhB = W.alloc<double>(nC * Vp);
        A.lhG = W.alloc<double>(nC * D * Vp); A.lhS = W.alloc<double>(nA * Vp);
        A.lGbNh = W.alloc<double>(nW * Vp); A.lGbh = W.alloc<double>(nW * Vp);
    }
    double* lmA = W.alloc<double>(9 * nC);
    double* lmB = W.alloc<double>(9 * nC);
    double* mC = W.alloc<double>(9 * nC);
    double* mF = W.alloc<double>(9 * nA);
    A.lmuC = W.alloc<double>(nC);
    A.lmuF = W.alloc<double>(nA);
    A.lTw = W.alloc<double>(nW);
    if (W.oom) return s.fail(DUGKS_ERR_OOM, "adjoint: device allocation failed (states)");
    // 1. forward with checkpoints
    fwd_init(s, f);
    for (int n = 0; n < N; ++n) {
        if (n % K == 0) save(ckpt + stateN * (size_t)(n / K));
        fwd_step(s, f, o, n, wq, ws, dJ);
    }
    cudaMemcpyAsync(&J, dJ, 8, cudaMemcpyDeviceToHost, st);
    // 2. reverse, segment by segment
    A.muRef = a.muRef;
    A.M = M;
    A.wq = wq;
    A.ws = ws;
    double* lmN = lmA;  // adjoint of the macros at n+1
    double* lm = lmB;
    for (int sg = nSeg - 1; sg >= 0; --sg) {
        const int n0 = sg * K, n1 = std::min(N, n0 + K);
        restore(ckpt + stateN * (size_t)sg);
        save(seg);
        for (int n = n0; n < n1; ++n) {
            if (inter) {
                fwd_step(s, f, o, n, nullptr, nullptr, nullptr, 4);  // P1..P6
                double* it = inter + interN * (size_t)(n - n0);
                cudaMemcpyAsync(it + iS, f.b.gS, nA * Vp * 8, cudaMemcpyDeviceToDevice, st);
                if (a.hasH) cudaMemcpyAsync(it + iSh, f.b.hS, nA * Vp * 8, cudaMemcpyDeviceToDevice, st);
                adj_pack_macros(a.nA, a.rhoF, a.UF, a.TF, a.qF, a.tauF, it + iF, sms, st);
                cudaMemcpyAsync(it + iW, a.rhoW, nW * 8, cudaMemcpyDeviceToDevice, st);
                fwd_step(s, f, o, n, nullptr, nullptr, nullptr, kRefKernels - 1, 5);  // P7..P9
            } else {
                fwd_step(s, f, o, n, nullptr, nullptr, nullptr);
            }
            save(seg + stateN * (size_t)(n - n0 + 1));
        }
        for (int n = n1 - 1; n >= n0; --n) {
            const double* stN = seg + stateN * (size_t)(n - n0);
            const double* stN1 = seg + stateN * (size_t)(n - n0 + 1);
            A.a = f.a;
            if (inter) {
                const double* it = inter + interN * (size_t)(n - n0);
                const double* m = stN + oM;
                adj_pack_macros(a.nC, m, m + nC, m + 4 * nC, m + 5 * nC, m + 8 * nC, mC, sms, st);
                A.gT = stN + oG; A.hT = a.hasH ? stN + oH : nullptr;
                A.gS = it + iS; A.hS = a.hasH ? it + iSh : nullptr;
                A.mF = it + iF;
                A.a.rhoW = const_cast<double*>(it + iW);
            } else {
                restore(stN);
                fwd_step(s, f, o, n, nullptr, nullptr, nullptr, 4);  // P1..P6 of step n
                adj_pack_macros(a.nC, a.rho, a.U, a.T, a.q, a.tau, mC, sms, st);
                adj_pack_macros(a.nA, a.rhoF, a.UF, a.TF, a.qF, a.tauF, mF, sms, st);
                A.gT = f.b.gT; A.hT = f.b.hT; A.gS = f.b.gS; A.hS = f.b.hS;
                A.mF = mF;
            }
            A.mC = mC;
            A.lmN = lmN; A.lm = lm;
            A.haveMacroAdj = n < N - 1;
            adj_launch_step(A, stN1 + oG, a.hasH ? stN1 + oH : nullptr, stN1 + oM, in_window(o, n), window_scale(o), sms,
                            st);
            std::swap(A.lgN, A.lgT);
            std::swap(A.lhN, A.lhT);
            std::swap(A.lGbN, A.lGb);
            std::swap(A.lGbNh, A.lGbh);
            std::swap(lmN, lm);
        }
    }
    // 3. parameter adjoints: mu from every tau (cells, faces, the initial tau0)
    double* dmu = W.alloc<double>(1);
    if (W.oom) return s.fail(DUGKS_ERR_OOM, "adjoint: device allocation failed");
    adj_sum(a.nC, A.lmuC, dmu, st);
    adj_sum(a.nA, A.lmuF, dmu, st);
    std::vector<double> lm0(9 * nC), tau0(nC);
    cudaMemcpyAsync(lm0.data(), lmN, 9 * nC * 8, cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(tau0.data(), ckpt + oM + 8 * nC, nC * 8, cudaMemcpyDeviceToHost, st);
    double hmu = 0.0;
    cudaMemcpyAsync(&hmu, dmu, 8, cudaMemcpyDeviceToHost, st);
    if (dJdTw && a.nW) cudaMemcpyAsync(dJdTw, A.lTw, a.nW * 8, cudaMemcpyDeviceToHost, st);
    if (int e = finish(s, "adjoint")) return e;
    for (size_t c = 0; c < nC; ++c) hmu += lm0[9 * c + 8] * tau0[c] / a.muRef;  // tau0 = tau(T0, rho0; mu)
    dJdMuScale = hmu * a.muRef;
    return DUGKS_OK;
}

}  // namespace dugks
