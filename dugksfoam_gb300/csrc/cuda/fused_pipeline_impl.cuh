// FusedPipelineT<S>: owns the tile plan and the double-buffered state of the
// fused step; included once per storage type (fused_fp32.cu, fused_fp64.cu).
// FP64: two tiled sweeps (fused_kernels.cuh).  FP32: face sides on one-ring
// tiles, face macros, cell gather (fused32.cuh).
#pragma once

#include <cmath>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "../host/solver.h"
#include "../host/tile_plan.h"
#include "fused32.cuh"
#include "fused_kernels.cuh"
#include "kernels.h"

namespace dugks {

template <typename S>
class FusedPipelineT final : public FusedPipeline {
public:
    using KernelFn = void (*)(FusedArgs<S>);

    ~FusedPipelineT() override {
        for (void* p : allocs_) cudaFree(p);
    }

    bool init(Solver& solver, const StepArgs& a, std::string& err) {
        const Mesh& m = solver.mesh();
        if (a.D != 2 && a.D != 3) { err = "the fused pipelines need a 2D or 3D mesh (1D runs on the plain FP64 pipeline)"; return false; }
        D_ = a.D;
        bcMask_ = a.bcMask;
        H_ = a.hasH != 0;
        if (D_ != 2 && D_ != 3) { err = "fused pipeline supports 2D and 3D meshes"; return false; }
        npl_ = fused_npl(sizeof(S) == 4 ? DUGKS_FP32_FP64MOM : DUGKS_FP64);
        fp32_ = sizeof(S) == 4;
        const int KC = 32 * npl_;
        if (a.Vp % KC != 0) { err = "padded DV count is not a multiple of the DV chunk"; return false; }
        // ---- tile plan, sized to the shared-memory budget
        int dev = 0;
        cudaGetDevice(&dev);
        int maxSmem = 0;
        cudaDeviceGetAttribute(&maxSmem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
        pick();
        const size_t budget = (size_t)maxSmem - 2048;
        const char* envT = std::getenv("DUGKS_TILE_CELLS");
        const int maxCells = fused_tile_cap() > 0 ? fused_tile_cap() : (envT ? std::max(1, std::atoi(envT)) : 4096);
        // FP32: sweep A alone is tiled (one-ring halo); FP64: both sweeps (two-ring halo)
        const SmemFn fn = [this](const TileDims& d) { return fp32_ ? smemFace(d) : std::max(smemFace(d), smemCell(d)); };
        // one tile per SM at a time: balance the waves of the FP32 face sweep,
        // unless a cap was asked for or the case's tiles share the batched
        // kernels' grid with other cases' tiles
        int nsmPlan = 0;
        cudaDeviceGetAttribute(&nsmPlan, cudaDevAttrMultiProcessorCount, dev);
        const int waveSlots = fp32_ && fused_wave_balance() && !envT ? nsmPlan : 0;
        if (!build_tile_plan(m, maxCells, fn, budget, plan_, err, fp32_ ? 1 : 2, waveSlots)) return false;
        smemA_ = smemB_ = 0;
        for (const TileHdr& h : plan_.hdr) {
            TileDims d;
            d.nT = h.nT; d.nT1 = h.nT1; d.nT2 = h.nT2; d.nFA = h.nFA; d.nFB = h.nFB; d.nEnt = h.nEnt;
            smemA_ = std::max(smemA_, smemFace(d));
            if (!fp32_) smemB_ = std::max(smemB_, smemCell(d));
        }
        // The limit is a property of the kernel function, shared by every
        // pipeline (case) that launches it: allow the device maximum, each
        // launch then asks for its own size.
        allow_max_dynamic_smem(kFace_);
        if (!fp32_) allow_max_dynamic_smem(kCell_);

        // ---- upload plan
        args_.hdr = upload(plan_.hdr);
        if (!fp32_) {  // the FP32 kernels read per-tile metadata blocks instead
            args_.cells = upload(plan_.cells);
            args_.faces = upload(plan_.faces);
            args_.colorOff = upload(plan_.colorOff);
            args_.colorPerm = upload(plan_.colorPerm);
        }
        const size_t nRec = plan_.faces.size();
        if (sizeof(S) == 4) {
            std::vector<float4> st4(plan_.stEnt.size());
            for (size_t e = 0; e < st4.size(); ++e) {
                int o = plan_.stEnt[e];
                float ow;
                std::memcpy(&ow, &o, 4);
                st4[e] = make_float4((float)plan_.stL[3 * e], (float)plan_.stL[3 * e + 1], (float)plan_.stL[3 * e + 2], ow);
            }
            std::vector<float4> fg4(3 * nRec);
            for (size_t k = 0; k < nRec; ++k) {
                const TileFace& r = plan_.faces[k];
                const int f = r.a < m.nI ? r.a : m.wallFace[r.a - m.nI];
                const int o = m.owner[f];
                double Sv[3], dO[3], dN[3] = {0, 0, 0};
                for (int q = 0; q < 3; ++q) {
                    Sv[q] = m.Sf[3 * (size_t)f + q];
                    dO[q] = m.Cf[3 * (size_t)f + q] - m.C[3 * (size_t)o + q];
                    if (r.a < m.nI) dN[q] = m.Cf[3 * (size_t)f + q] - m.C[3 * (size_t)m.neighbour[f] + q];
                    else dN[q] = m.nHatW[3 * (size_t)r.w + q];  // wall: unit normal
                }
                const double iVo = 1.0 / m.V[o], iVn = r.a < m.nI ? 1.0 / m.V[m.neighbour[f]] : 0.0;
                fg4[3 * k] = make_float4((float)Sv[0], (float)Sv[1], (float)Sv[2], (float)iVo);
                fg4[3 * k + 1] = make_float4((float)dO[0], (float)dO[1], (float)dO[2], (float)iVn);
                // plain-stencil code: entries of each side when every one is
                // a cell row (no wall entry), else 0; owner | neighbour << 8
                auto plainN = [&](int e0, int e1) {
                    for (int e = e0; e < e1; ++e)
                        if (plan_.stEnt[e] < 0) return 0;
                    return std::min(e1 - e0, 255);
                };
                const int plain = plainN(r.stO0, r.stO1) | (r.neiL >= 0 ? plainN(r.stN0, r.stN1) << 8 : 0);
                float pw;
                std::memcpy(&pw, &plain, 4);
                fg4[3 * k + 2] = make_float4((float)dN[0], (float)dN[1], (float)dN[2], pw);
            }
            // per-tile blocks: face records (stencil ranges relative to the
            // tile's first entry) + geometry, entries, cells, colour order
            std::vector<int4> meta;
            std::vector<int> metaOff;
            auto ints = [&](const int32_t* v, int n) {
                for (int i = 0; i < n; i += 4)
                    meta.push_back(make_int4(v[i], i + 1 < n ? v[i + 1] : 0, i + 2 < n ? v[i + 2] : 0,
                                             i + 3 < n ? v[i + 3] : 0));
            };
            auto f4i = [](float4 f) {
                int4 r;
                std::memcpy(&r, &f, 16);
                return r;
            };
            for (const TileHdr& h : plan_.hdr) {
                metaOff.push_back((int)meta.size());
                const int base = plan_.stOff[h.stStart];
                for (int k = 0; k < h.nFB; ++k) {
                    const size_t rec = (size_t)h.faceStart + k;
                    const TileFace& r = plan_.faces[rec];
                    meta.push_back(make_int4(r.ownL, r.neiL, r.a, r.w));
                    const bool so = r.stO1 > r.stO0, sn = r.neiL >= 0 && r.stN1 > r.stN0;  // non-empty stencils
                    meta.push_back(make_int4(so ? r.stO0 - base : 0, so ? r.stO1 - base : 0, sn ? r.stN0 - base : 0,
                                             sn ? r.stN1 - base : 0));
                    for (int q = 0; q < 3; ++q) meta.push_back(f4i(fg4[3 * rec + q]));
                }
                for (int e = 0; e < h.nEnt; ++e) meta.push_back(f4i(st4[(size_t)base + e]));
                ints(&plan_.cells[h.cellStart], h.nT2);
                std::vector<int32_t> cst(h.nT + 1);  // T cells' stencil ranges, tile-relative
                for (int i = 0; i <= h.nT; ++i) cst[i] = plan_.stOff[h.stStart + i] - base;
                ints(cst.data(), h.nT + 1);
                const int n16 = (int)meta.size() - metaOff.back();
                if (n16 > tile_meta32_bound(h.nFB, h.nEnt, h.nT2)) { err = "tile metadata exceeds its bound"; return false; }
            }
            metaOff.push_back((int)meta.size());
            args_.meta = upload(meta);
            args_.metaOff = upload(metaOff);
            {
                // faces of each cell in global face order, S oriented out of the cell
                std::vector<int> cfOff(m.nC + 1);
                std::vector<float4> cfEnt;
                for (int c = 0; c < m.nC; ++c) {
                    cfOff[c] = (int)cfEnt.size();
                    for (int j = m.cellOff[c]; j < m.cellOff[c + 1]; ++j) {
                        const int af = m.cellFace[j];
                        const int gf = af < m.nI ? af : m.wallFace[af - m.nI];
                        const double sg = m.cellSide[j] == 0 ? 1.0 : -1.0;
                        float code;
                        std::memcpy(&code, &af, 4);
                        cfEnt.push_back(make_float4((float)(sg * m.Sf[3 * (size_t)gf]), (float)(sg * m.Sf[3 * (size_t)gf + 1]),
                                                    (float)(sg * m.Sf[3 * (size_t)gf + 2]), code));
                    }
                }
                cfOff[m.nC] = (int)cfEnt.size();
                for (int c = 0; c < m.nC; ++c) gatherMF_ = std::max(gatherMF_, cfOff[c + 1] - cfOff[c]);
                gatherMF_ = std::min(gatherMF_, 8);  // further faces of a cell are read directly
                gatherSmem_ = gather_smem(kGatherWarps, gatherMF_, KC, H_);
                allow_max_dynamic_smem(kGather_);
                int per = 0, nsm = 0;
                cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kGather_, kGatherWarps * 32, gatherSmem_);
                // the velocity constants in shared memory when they are small
                // (2D grids up to 1536 padded velocities: <= 24 KB per block)
                // and the blocks per SM stay as they are without them
                if (fp32_ && D_ == 2 && dv_table32_bytes(D_, a.Vp) <= 24 * 1024) {
                    int perTab = 0;
                    const size_t withTab = gatherSmem_ + dv_table32_bytes(D_, a.Vp);
                    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perTab, kGather_, kGatherWarps * 32, withTab);
                    if (perTab >= per) {
                        gatherTab_ = true;
                        gatherSmem_ = withTab;
                        per = perTab;
                    }
                }
                cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
                gatherBlocks_ = std::max(1, per) * std::max(1, nsm);  // persistent: one wave
                args_.cfOff = upload(cfOff);
                args_.cfEnt = upload(cfEnt);
                std::vector<float> iv(m.nC);
                for (int c = 0; c < m.nC; ++c) iv[c] = (float)(1.0 / m.V[c]);
                args_.invVf = upload(iv);
                args_.gF = alloc<float>((size_t)a.nA * a.Vp);
                args_.hF = H_ ? alloc<float>((size_t)a.nA * a.Vp) : nullptr;
                args_.feqT = alloc<float4>(3 * (size_t)a.nA);
                args_.faceMom = alloc<double>((size_t)a.nA * 2 * 32);
            }
            std::vector<float4> w4(std::max(a.nW, 1), make_float4(0, 0, 0, 0));
            std::vector<double> Tw(a.nW);
            if (a.nW) cudaMemcpy(Tw.data(), a.Tw, a.nW * 8, cudaMemcpyDeviceToHost);
            for (int w = 0; w < a.nW; ++w) {
                // .y: 1/deltaCoeff of the lagged-gradient boundary value; 0 on
                // symmetryPlane (a constraint patch of gbar+: value = internal value)
                // .z: 0 wall, 1 open boundary, 2 symmetryPlane (relaxed twice outgoing)
                const int kind = m.wallKind[w];
                const bool plane = kind == DUGKS_PATCH_SYMMETRY_PLANE;
                w4[w] = make_float4((float)((a.R * Tw[w]) * (a.K + 3 - a.D)), plane ? 0.f : (float)(1.0 / m.dcW[w]),
                                    kind == DUGKS_PATCH_MAXWELL ? 0.f : (plane ? 2.f : 1.f), 0.f);
            }
            args_.wall4 = upload(w4);
            if (a.bcMask & ((1 << kBcSymmetryMod) | (1 << kBcSymmetryPlane))) {
                args_.symG = alloc<float>((size_t)a.nW * a.Vp);
                args_.symH = H_ ? alloc<float>((size_t)a.nW * a.Vp) : nullptr;
            }
            args_.rhoWs = alloc<float>(std::max(a.nW, 1));
            args_.uref4 = alloc<float4>(a.nA);
        } else {
            args_.stEnt = upload(plan_.stEnt);
            args_.stL = upload(plan_.stL);
            std::vector<double> fgeo(9 * nRec);
            for (size_t k = 0; k < nRec; ++k) {
                const TileFace& r = plan_.faces[k];
                const int f = r.a < m.nI ? r.a : m.wallFace[r.a - m.nI];
                const int o = m.owner[f];
                for (int q = 0; q < 3; ++q) {
                    fgeo[9 * k + q] = m.Sf[3 * (size_t)f + q];
                    fgeo[9 * k + 3 + q] = m.Cf[3 * (size_t)f + q] - m.C[3 * (size_t)o + q];
                    fgeo[9 * k + 6 + q] =
                        r.a < m.nI ? m.Cf[3 * (size_t)f + q] - m.C[3 * (size_t)m.neighbour[f] + q] : 0.0;
                }
            }
            args_.fgeo = upload(fgeo);
        }
        // ---- DV arrays in storage precision
        std::vector<double> xh(3 * (size_t)a.Vp), wh(a.Vp);
        cudaMemcpy(xh.data(), a.xi, xh.size() * 8, cudaMemcpyDeviceToHost);
        cudaMemcpy(wh.data(), a.w, wh.size() * 8, cudaMemcpyDeviceToHost);
        args_.xi = upload(std::vector<S>(xh.begin(), xh.end()));
        args_.w = upload(std::vector<S>(wh.begin(), wh.end()));
        // ---- state
        const size_t nCV = (size_t)a.nC * a.Vp, nWV = (size_t)std::max(a.nW, 1) * a.Vp;
        for (int i = 0; i < 2; ++i) {
            gT_[i] = alloc<S>(nCV);
            hT_[i] = H_ ? alloc<S>(nCV) : nullptr;
            Gg_[i] = alloc<S>(nWV);
            Gh_[i] = H_ ? alloc<S>(nWV) : nullptr;
            cc_[i] = sizeof(S) == 4 ? alloc<float>((size_t)a.nC * kNCoef) : nullptr;
        }
        args_.Mw = mw_ = alloc<S>(nWV);
        min_ = alloc<double>((size_t)std::max(a.nW, 1) * 32);
        args_.Min = min_;
        args_.fc = sizeof(S) == 4 ? alloc<float>((size_t)a.nA * kNCoef) : nullptr;
        if (sizeof(S) == 4) {
            mref_ = alloc<float>(a.Vp);
            refMom_ = alloc<double>(32);
            wallRefOut_ = alloc<double>((size_t)std::max(a.nW, 1) * 32);
            args_.mref = mref_;
            args_.refMom = refMom_;
            args_.wallRefOut = wallRefOut_;
        }
        rhoN_ = alloc<double>(a.nC); UN_ = alloc<double>(3 * (size_t)a.nC); TN_ = alloc<double>(a.nC);
        qN_ = alloc<double>(3 * (size_t)a.nC); tauN_ = alloc<double>(a.nC);
        if (oom_) { err = "fused pipeline: device allocation failed"; return false; }
        // density scale of the stored distributions: O(1) values in FP32
        if (sizeof(S) == 4) {
            std::vector<double> r0(a.nC), t0(a.nC);
            cudaMemcpy(r0.data(), a.rho, a.nC * 8, cudaMemcpyDeviceToHost);
            cudaMemcpy(t0.data(), a.T, a.nC * 8, cudaMemcpyDeviceToHost);
            double rs = 0, ts = 0;
            for (int c = 0; c < a.nC; ++c) { rs += r0[c]; ts += t0[c]; }
            rs /= a.nC; ts /= a.nC;
            gscale_ = std::pow(2.0 * 3.14159265358979323846 * a.R * ts, 0.5 * D_) / rs;
            T0_ = ts;
            hrefFac_ = a.R * ts * (a.K + 3 - a.D);
            args_.hrefFac = (float)hrefFac_;
        } else {
            gscale_ = 1.0;
        }
        args_.gscale = gscale_;
        args_.invGscale = 1.0 / gscale_;
        return true;
    }

    double gscale() const override { return gscale_; }

    void initState(const StepArgs& a, int sms, cudaStream_t s) override {
        if constexpr (sizeof(S) == 4) {
            kRef_<<<1 + a.nW, 128, 0, s>>>(a, T0_, hrefFac_, mref_, refMom_, wallRefOut_);
            k_init_dev32<<<sms * 8, 256, 0, s>>>(a, mref_, gscale_, hrefFac_, gT_[0], hT_[0]);
        } else {
            launch_init_state<S>(a, gT_[0], hT_[0], gscale_, sms, s);
        }
        if (sizeof(S) == 4) {
            if (D_ == 2) k_cell_coef<2><<<sms * 4, 256, 0, s>>>(a, cc_[0], gscale_);
            else k_cell_coef<3><<<sms * 4, 256, 0, s>>>(a, cc_[0], gscale_);
        }
        if (a.nW > 0) kTables_<<<a.nW, 128, 0, s>>>(a, mw_, min_);
        if (sizeof(S) == 4) k_face_uref<<<sms * 2, 256, 0, s>>>(a, args_.uref4);
    }

    int nKernels() const override { return fp32_ ? 3 : 2; }
    const char* kernelName(int k) const override {
        if (fp32_) return k == 0 ? "k_face_sides" : (k == 1 ? "k_face_macros" : "k_cell_gather");
        return k == 0 ? "k_sweep_face" : "k_sweep_cell";
    }

    // Arguments of the step `parity` steps ahead (0: this step, 1: the next).
    FusedArgs<S> stepArgs(const StepArgs& a, int parity) const {
        FusedArgs<S> A = args_;
        A.b = a;
        A.dt = (S)a.dt;
        const int c = (cur_ + parity) & 1;
        A.gT = gT_[c]; A.hT = hT_[c];
        A.gTn = gT_[1 - c]; A.hTn = hT_[1 - c];
        A.Gbg = Gg_[c]; A.Gbh = Gh_[c];
        A.Gbgn = Gg_[1 - c]; A.Gbhn = Gh_[1 - c];
        A.cc = cc_[c]; A.ccn = cc_[1 - c];
        A.rhoN = rhoN_; A.UN = UN_; A.TN = TN_; A.qN = qN_; A.tauN = tauN_;
        if (parity & 1) {  // endStep swaps the cell macros into the base arguments
            std::swap(A.b.rho, A.rhoN); std::swap(A.b.U, A.UN); std::swap(A.b.T, A.TN);
            std::swap(A.b.q, A.qN); std::swap(A.b.tau, A.tauN);
        }
        return A;
    }

    bool batchable() const override { return fp32_; }
    bool batchKernels() const override { return fp32_ && (bcMask_ & ~(1 << kBcMaxwell)) == 0; }
    void batchArgs(const StepArgs& a, int parity, void* out) const override {
        const FusedArgs<S> A = stepArgs(a, parity);
        std::memcpy(out, &A, sizeof(A));
    }
    size_t batchArgsBytes() const override { return sizeof(FusedArgs<S>); }
    int batchTiles() const override { return plan_.nTiles; }
    size_t batchSmemFace() const override { return smemA_; }
    int batchGatherMF() const override { return gatherMF_; }
    int batchNpl() const override { return npl_; }

    void launchParity(const StepArgs& a, int parity, int sms, cudaStream_t s) override {
        for (int k = 0; k < nKernels(); ++k) launchArgs(k, stepArgs(a, parity), a, sms, s);
    }

    void launch(int k, const StepArgs& a, int sms, cudaStream_t s) override { launchArgs(k, stepArgs(a, 0), a, sms, s); }

    void launchArgs(int k, const FusedArgs<S>& A, const StepArgs& a, int sms, cudaStream_t s) {
        (void)sms;
        if (k == 0) {
            kFace_<<<plan_.nTiles, kWarps * 32, smemA_, s>>>(A);
            if (kOpen_) kOpen_<<<std::max(1, std::min((a.nW + 3) / 4, sms * 8)), 128, 0, s>>>(A);
        }
        else if (!fp32_) kCell_<<<plan_.nTiles, kWarps * 32, smemB_, s>>>(A);
        else if (k == 1) kMacros_<<<std::max(1, (a.nA + 127) / 128), 128, 0, s>>>(A);  // one face per thread
        else {
            kGather_<<<std::min((a.nC + kGatherWarps - 1) / kGatherWarps, gatherBlocks_), kGatherWarps * 32, gatherSmem_,
                       s>>>(A, gatherMF_, gatherTab_ ? 1 : 0);
            if (a.zgMask || (a.bcMask & ((1 << kBcPressureIn) | (1 << kBcPressureOut)))) {
                StepArgs n = A.b;  // zeroGradient U/T patches, then P10, from the macros this step wrote
                n.rho = A.rhoN; n.U = A.UN; n.T = A.TN;
                launch_zero_gradient_tu(n, s);
                if (a.bcMask & ((1 << kBcPressureIn) | (1 << kBcPressureOut))) launch_pressure_bc(n, s);
            }
        }
    }

    void endStep(StepArgs& base) override {
        cur_ = 1 - cur_;
        std::swap(base.rho, rhoN_);
        std::swap(base.U, UN_);
        std::swap(base.T, TN_);
        std::swap(base.q, qN_);
        std::swap(base.tau, tauN_);
    }

    void refreshDerived(const StepArgs& a, int sms, cudaStream_t s) override {
        if (sizeof(S) == 4) {
            if (D_ == 2) k_cell_coef<2><<<sms * 4, 256, 0, s>>>(a, cc_[cur_], gscale_);
            else k_cell_coef<3><<<sms * 4, 256, 0, s>>>(a, cc_[cur_], gscale_);
            k_face_uref<<<sms * 2, 256, 0, s>>>(a, args_.uref4);
        }
    }

    void exportDist(const StepArgs& a, int which, double* dst, int sms, cudaStream_t s) override {
        if constexpr (sizeof(S) == 4)
            k_export_dev32<<<sms * 8, 256, 0, s>>>(a, which ? hT_[cur_] : gT_[cur_], mref_, which ? hrefFac_ : 1.0,
                                                   1.0 / gscale_, dst);
        else
            launch_export_dist<S>(a, which ? hT_[cur_] : gT_[cur_], dst, 1.0 / gscale_, sms, s);
    }
    void importDist(const StepArgs& a, int which, const double* src, int sms, cudaStream_t s) override {
        if constexpr (sizeof(S) == 4)
            k_import_dev32<<<sms * 8, 256, 0, s>>>(a, src, mref_, which ? hrefFac_ : 1.0, gscale_,
                                                   which ? hT_[cur_] : gT_[cur_]);
        else
            launch_import_dist<S>(a, src, which ? hT_[cur_] : gT_[cur_], gscale_, sms, s);
    }
    void* distPtr(int which) override { return which ? (void*)hT_[cur_] : (void*)gT_[cur_]; }
    void* gradBPtr(int which) override { return which ? (void*)Gh_[cur_] : (void*)Gg_[cur_]; }
    size_t bytes() const override { return bytes_; }
    std::string describe() const override {
        char buf[256];
        snprintf(buf, sizeof(buf), "tiles=%d maxT=%d meanT=%.1f halo=%.2f maxT2=%d maxFB=%d npl=%d grad=%d smemA=%zu smemB=%zu gatherMF=%d",
                 plan_.nTiles, plan_.maxT, (double)plan_.sumT / std::max(1, plan_.nTiles),
                 (double)plan_.sumT2 / std::max(1LL, plan_.sumT), plan_.maxT2, plan_.maxFB, npl_, (int)grad_, smemA_, smemB_, gatherMF_);
        return buf;
    }

private:
    static constexpr int kWarps = 16;       // warps per tile block (one tile per SM)
    static constexpr int kGatherWarps = 8;  // warps (cells) per block of the gather sweep

    template <typename T>
    T* alloc(size_t n) {
        void* p = nullptr;
        const size_t by = std::max<size_t>(n, 1) * sizeof(T);
        if (cudaMalloc(&p, by) != cudaSuccess) { cudaGetLastError(); oom_ = true; return nullptr; }
        cudaMemset(p, 0, by);
        allocs_.push_back(p);
        bytes_ += by;
        return static_cast<T*>(p);
    }
    template <typename T>
    T* upload(const std::vector<T>& v) {
        T* p = alloc<T>(v.size());
        if (p && !v.empty()) cudaMemcpy(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice);
        return p;
    }

    template <int D, bool H, int NPL>
    void set() {
        if constexpr (sizeof(S) == 4) {
            // 3D: per-cell gradients once per chunk (six stencil entries a side, three faces a cell)
            grad_ = D == 3 || fused_face_grad();
            kFace_ = grad_ ? k_face_sides32<D, H, NPL, kWarps, true> : k_face_sides32<D, H, NPL, kWarps, false>;
            kMacros_ = k_face_macros32<D, H>;
            kOpen_ = (bcMask_ & ~(1 << kBcMaxwell)) ? k_open_faces32<D, H, NPL> : nullptr;
            kGather_ = (bcMask_ & ~(1 << kBcMaxwell)) ? k_cell_gather32<D, H, NPL, kGatherWarps, true>
                                                     : k_cell_gather32<D, H, NPL, kGatherWarps, false>;
            kRef_ = k_ref_tables<D, H>;
        } else {
            kFace_ = k_sweep_face<S, D, H, NPL, kWarps>;
            kCell_ = k_sweep_cell<S, D, H, NPL, kWarps>;
        }
        kTables_ = k_wall_tables<S, D, H>;
        if constexpr (sizeof(S) == 4) {
            smemFaceFn_ = grad_ ? &SmemLayout32<D, H, NPL, true>::sides : &SmemLayout32<D, H, NPL, false>::sides;
            smemCellFn_ = nullptr;
        } else {
            smemFaceFn_ = &SmemLayout<S, D, H, NPL>::face;
            smemCellFn_ = &SmemLayout<S, D, H, NPL>::cell;
        }
    }
    template <int D, bool H>
    void setD() {
        if constexpr (sizeof(S) == 4) {
            if (npl_ == 4) set<D, H, 4>();
            else set<D, H, 2>();
        } else {
            set<D, H, 1>();
        }
    }
    void pick() {
        if (D_ == 2) { H_ ? setD<2, true>() : setD<2, false>(); }
        else { H_ ? setD<3, true>() : setD<3, false>(); }
    }
    size_t smemFace(const TileDims& d) const { return smemFaceFn_(d); }
    size_t smemCell(const TileDims& d) const { return smemCellFn_(d); }

    int D_ = 2, npl_ = 1;
    bool fp32_ = false, grad_ = false;
    int bcMask_ = 1 << kBcMaxwell;
    KernelFn kMacros_ = nullptr;
    KernelFn kOpen_ = nullptr;  // open boundary faces after sweep A (when the case has any)
    int gatherMF_ = 0, gatherBlocks_ = 1;
    bool gatherTab_ = false;
    size_t gatherSmem_ = 0;
    void (*kGather_)(FusedArgs<S>, int, int) = nullptr;
    bool H_ = true;
    TilePlan plan_;
    FusedArgs<S> args_{};
    KernelFn kFace_ = nullptr, kCell_ = nullptr;
    void (*kTables_)(StepArgs, S*, double*) = nullptr;
    void (*kRef_)(StepArgs, double, double, float*, double*, double*) = nullptr;
    float* mref_ = nullptr;
    double* refMom_ = nullptr;
    double* wallRefOut_ = nullptr;
    double T0_ = 273.0, hrefFac_ = 0.0;
    size_t (*smemFaceFn_)(const TileDims&) = nullptr;
    size_t (*smemCellFn_)(const TileDims&) = nullptr;
    size_t smemA_ = 0, smemB_ = 0;
    S* gT_[2] = {nullptr, nullptr};
    S* hT_[2] = {nullptr, nullptr};
    S* Gg_[2] = {nullptr, nullptr};
    S* Gh_[2] = {nullptr, nullptr};
    float* cc_[2] = {nullptr, nullptr};
    S* mw_ = nullptr;
    double* min_ = nullptr;
    double *rhoN_ = nullptr, *UN_ = nullptr, *TN_ = nullptr, *qN_ = nullptr, *tauN_ = nullptr;
    double gscale_ = 1.0;
    int cur_ = 0;
    std::vector<void*> allocs_;
    size_t bytes_ = 0;
    bool oom_ = false;
};

}  // namespace dugks
