// The two fused sweep kernels and their set-up kernels (see fused_impl.cuh).
#pragma once

#include "fused_impl.cuh"

namespace dugks {

template <typename S, int D, bool H, int NPL>
struct SmemLayout {
    static constexpr int KC = 32 * NPL;
    static constexpr int NS = Slots<D, H>::NS;
    __host__ __device__ static size_t rows(int n) { return (size_t)n * KC * sizeof(S) * (H ? 2 : 1); }
    __host__ __device__ static size_t align(size_t x) { return (x + 15) & ~size_t(15); }
    static size_t face(const TileDims& d) { return align(rows(d.nT2)) + (size_t)d.nFA * NS * sizeof(Acc<S>); }
    static size_t cell(const TileDims& d) {
        return align(rows(d.nT2)) + align(rows(d.nT)) + (size_t)d.nT * NS * sizeof(Acc<S>);
    }
};

// DV constants of the lane's NPL velocities in the current chunk.
template <typename S, int D, int NPL>
struct LaneDV {
    S xi[NPL][3];
    S w[NPL];
    __device__ __forceinline__ void load(const FusedArgs<S>& A, int v0, int lane) {
        const int Vp = A.b.Vp;
#pragma unroll
        for (int j = 0; j < NPL; ++j) {
            const int v = v0 + j * 32 + lane;
            xi[j][0] = A.xi[v];
            xi[j][1] = A.xi[Vp + v];
            xi[j][2] = D == 3 ? A.xi[2 * Vp + v] : S(0);
            w[j] = A.w[v];
        }
    }
};

// gbar+ rows (and, for sweep B, the -1/3 g~ + 4/3 gbar+ partial of T's rows).
template <typename S, int D, bool H, int NPL, int NW, bool PARTIAL>
__device__ __forceinline__ void stage_rows(const FusedArgs<S>& A, const TileHdr& hd, const LaneDV<S, D, NPL>& dv,
                                           int v0, int lane, int warp, S* sg, S* sh, S* sa, S* sah) {
    constexpr int KC = 32 * NPL;
    const int Vp = A.b.Vp;
    for (int lc = warp; lc < hd.nT2; lc += NW) {
        const int c = A.cells[hd.cellStart + lc];
        Relax<S, D, H> rx;
        rx.loadCell(A, c);
        S g0[NPL], h0[NPL];
#pragma unroll
        for (int j = 0; j < NPL; ++j) {
            const size_t gi = (size_t)c * Vp + v0 + j * 32 + lane;
            g0[j] = A.gT[gi];
            h0[j] = H ? A.hT[gi] : S(0);
        }
#pragma unroll
        for (int j = 0; j < NPL; ++j) {
            const int col = j * 32 + lane;
            S g = g0[j], h = h0[j];
            rx.apply(dv.xi[j], g, h);
            sg[lc * KC + col] = g;
            if (H) sh[lc * KC + col] = h;
            if (PARTIAL && lc < hd.nT) {
                if constexpr (sizeof(S) == 8) {  // reference order (discreteVelocity.C:938-939)
                    sa[lc * KC + col] = -1.0 / 3 * g0[j] + 4.0 / 3 * g;
                    if (H) sah[lc * KC + col] = -1.0 / 3 * h0[j] + 4.0 / 3 * h;
                } else {  // g+ + (g+ - g~)/3: exact when g+ == g~ (no FP32 mass bias)
                    sa[lc * KC + col] = fmaf(g - g0[j], 1.0f / 3.0f, g);
                    if (H) sah[lc * KC + col] = fmaf(h - h0[j], 1.0f / 3.0f, h);
                }
            }
        }
    }
}

// ---------------------------------------------------------------- sweep A
template <typename S, int D, bool H, int NPL, int NW>
__global__ void __launch_bounds__(NW * 32, 1) k_sweep_face(FusedArgs<S> A) {
    using SL = Slots<D, H>;
    using LY = SmemLayout<S, D, H, NPL>;
    constexpr int NS = SL::NS, KC = LY::KC;
    extern __shared__ __align__(16) unsigned char smem[];
    const TileHdr hd = A.hdr[blockIdx.x];
    const StepArgs& b = A.b;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int Vp = b.Vp;
    S* sg = reinterpret_cast<S*>(smem);
    S* sh = sg + (size_t)hd.nT2 * KC;
    Acc<S>* mom = reinterpret_cast<Acc<S>*>(smem + LY::align(LY::rows(hd.nT2)));
    for (int i = threadIdx.x; i < hd.nFA * NS; i += NW * 32) mom[i].zero();
    const int nChunks = Vp / KC;
    const int myslot = slot_of<NS>(lane);
    const bool writer = NS == 16 ? (lane & 1) == 0 : true;

    for (int ch = 0; ch < nChunks; ++ch) {
        const int v0 = ch * KC;
        LaneDV<S, D, NPL> dv;
        dv.load(A, v0, lane);
        __syncthreads();
        stage_rows<S, D, H, NPL, NW, false>(A, hd, dv, v0, lane, warp, sg, sh, nullptr, nullptr);
        __syncthreads();
        for (int lf = warp; lf < hd.nFA; lf += NW) {
            const TileFace r = A.faces[hd.faceStart + lf];
            FaceGeo<S> fg;
            fg.load(A, hd.faceStart + lf);
            S ur[3];
            if constexpr (sizeof(S) == 4) {
                const float4 u4 = A.uref4[r.a];
                ur[0] = u4.x; ur[1] = u4.y; ur[2] = u4.z;
            } else {
                const double* urd = r.w >= 0 ? b.Uw + 3 * r.w : b.UF + 3 * r.a;
                ur[0] = urd[0]; ur[1] = urd[1]; ur[2] = urd[2];
            }
            S m[NS];
#pragma unroll
            for (int s = 0; s < NS; ++s) m[s] = S(0);
#pragma unroll
            for (int j = 0; j < NPL; ++j) {
                const int col = j * 32 + lane, v = v0 + col;
                const S* xi = dv.xi[j];
                S xs = S(0);
#pragma unroll
                for (int k = 0; k < D; ++k) xs += xi[k] * fg.Sv[k];
                S gf = S(0), hf = S(0);
                bool have;
                if (r.w >= 0) {
                    // lagged fixedGradient gradient G_b = grad(gbar+)_P . n for the next step
                    S gg[D], hg[D];
                    const S gc = sg[r.ownL * KC + col], hc = H ? sh[r.ownL * KC + col] : S(0);
                    stencil_grad<S, D, H>(A, r.stO0, r.stO1, gc, hc, sg, sh, KC, col, v, gg, hg);
                    S nh[3];
                    if constexpr (sizeof(S) == 4) {
                        nh[0] = fg.dN[0]; nh[1] = fg.dN[1]; nh[2] = fg.dN[2];
                    } else {
                        const double* n = b.nHatW + 3 * r.w;
                        nh[0] = n[0]; nh[1] = n[1]; nh[2] = n[2];
                    }
                    S sgn = S(0), shn = S(0);
#pragma unroll
                    for (int k = 0; k < D; ++k) { sgn += gg[k] * nh[k]; if (H) shn += hg[k] * nh[k]; }
                    A.Gbgn[(size_t)r.w * Vp + v] = sgn;
                    if (H) A.Gbhn[(size_t)r.w * Vp + v] = shn;
                    have = xs > S(0);
                    if (have) {
                        gf = recon<S, D>(gc, gg, fg.dO, xi, A.dt);
                        if (H) hf = recon<S, D>(hc, hg, fg.dO, xi, A.dt);
                        m[SL::FLUX] += dv.w[j] * xs * gf;
                    }
                } else {
                    have = face_value<S, D, H>(A, r, fg, sg, sh, KC, col, v, xi, xs, gf, hf);
                }
                if (have) {
                    S c[3];
#pragma unroll
                    for (int k = 0; k < D; ++k) c[k] = xi[k] - ur[k];
                    add_moments<S, D, H, NS, S>(m, dv.w[j], gf, hf, c);
                }
            }
            const S tot = reduce_scatter<NS, S>(m, lane);
            if (writer && myslot <= SL::FLUX) mom[lf * NS + myslot].add(tot);
        }
    }
    __syncthreads();
    // ---- finalize owned faces (FP64): Maxwell-wall density, face macros
    for (int lf = threadIdx.x; lf < hd.nFA; lf += NW * 32) {
        const TileFace r = A.faces[hd.faceStart + lf];
        double M[NS];
        for (int s = 0; s < NS; ++s) M[s] = mom[lf * NS + s].value();
        double ur[3];
        if constexpr (sizeof(S) == 4) {
            const float4 u4 = A.uref4[r.a];
            ur[0] = u4.x; ur[1] = u4.y; ur[2] = u4.z;
        } else {
            const double* urd = r.w >= 0 ? b.Uw + 3 * r.w : b.UF + 3 * r.a;
            for (int k = 0; k < 3; ++k) ur[k] = urd[k];
        }
        double rw = 0.0;
        if (r.w >= 0) {
            rw = M[SL::FLUX] / b.incAbs[r.w];
            for (int s = 0; s < SL::NM; ++s) M[s] += rw * A.Min[(size_t)r.w * NS + s];
        }
        for (int s = 0; s < SL::NM; ++s) M[s] *= A.invGscale;
        double rho, U[3], T, tau, qr[3];
        macros_from_moments<D, H>(M, ur, b, rho, U, T, tau, qr);
        const double fac = 2.0 * tau / (2.0 * tau + 0.5 * b.dt * b.Pr);
        double q[3] = {fac * qr[0], fac * qr[1], fac * qr[2]};
        const int a = r.a;
        b.rhoF[a] = rho;
        b.TF[a] = T;
        b.tauF[a] = tau;
        for (int k = 0; k < 3; ++k) { b.UF[3 * a + k] = U[k]; b.qF[3 * a + k] = q[k]; }
        if constexpr (sizeof(S) == 4) {
            write_coef<D>(A.fc + (size_t)a * kNCoef, rho, U, T, q, tau, b, A.gscale);
            if (r.w < 0) A.uref4[a] = make_float4((float)U[0], (float)U[1], (float)U[2], 0.0f);
        }
        if (r.w >= 0) {
            const int w = r.w;
            b.rhoW[w] = rw * A.invGscale;
            if constexpr (sizeof(S) == 4) A.rhoWs[w] = (float)rw;
            const double fq = 2.0 * tau / (2.0 * tau + 0.5 * b.dt * b.Pr);
            const double fs = 2.0 * tau / (2.0 * tau + 0.5 * b.dt);
            for (int k = 0; k < 3; ++k) {
                double v = 0.0;
                if (k < D) v = 0.5 * M[SL::M3 + k] + (H ? 0.5 * M[SL::H1 + k] : 0.0);
                b.qWall[3 * w + k] = fq * v;
            }
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j) {
                    double s = 0.0;
                    if (i < D && j < D) {
                        const double m2 = M[SL::M2 + (i <= j ? sym<D>(i, j) : sym<D>(j, i))];
                        s = m2 + ur[i] * M[SL::M1 + j] + ur[j] * M[SL::M1 + i] + ur[i] * ur[j] * M[0];
                    }
                    b.stressWall[9 * w + 3 * i + j] = fs * s;
                }
        }
    }
}

// ---------------------------------------------------------------- sweep B
template <typename S, int D, bool H, int NPL, int NW>
__global__ void __launch_bounds__(NW * 32, 1) k_sweep_cell(FusedArgs<S> A) {
    using SL = Slots<D, H>;
    using LY = SmemLayout<S, D, H, NPL>;
    constexpr int NS = SL::NS, KC = LY::KC;
    extern __shared__ __align__(16) unsigned char smem[];
    const TileHdr hd = A.hdr[blockIdx.x];
    const StepArgs& b = A.b;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int Vp = b.Vp;
    S* sg = reinterpret_cast<S*>(smem);
    S* sh = sg + (size_t)hd.nT2 * KC;
    S* sa = reinterpret_cast<S*>(smem + LY::align(LY::rows(hd.nT2)));
    S* sah = sa + (size_t)hd.nT * KC;
    Acc<S>* mom = reinterpret_cast<Acc<S>*>(smem + LY::align(LY::rows(hd.nT2)) + LY::align(LY::rows(hd.nT)));
    for (int i = threadIdx.x; i < hd.nT * NS; i += NW * 32) mom[i].zero();
    const int nChunks = Vp / KC;
    const int myslot = slot_of<NS>(lane);
    const bool writer = NS == 16 ? (lane & 1) == 0 : true;

    for (int ch = 0; ch < nChunks; ++ch) {
        const int v0 = ch * KC;
        LaneDV<S, D, NPL> dv;
        dv.load(A, v0, lane);
        __syncthreads();
        stage_rows<S, D, H, NPL, NW, true>(A, hd, dv, v0, lane, warp, sg, sh, sa, sah);
        __syncthreads();
        for (int ci = 0; ci < hd.nColors; ++ci) {
            const int k0 = A.colorOff[hd.colStart + ci], k1 = A.colorOff[hd.colStart + ci + 1];
            for (int k = k0 + warp; k < k1; k += NW) {
                const int lf = A.colorPerm[hd.permStart + k];
                const TileFace r = A.faces[hd.faceStart + lf];
                FaceGeo<S> fg;
                fg.load(A, hd.faceStart + lf);
                Relax<S, D, H> rf;
                rf.loadFace(A, r.a);
                const bool ownIn = r.ownL < hd.nT, neiIn = r.neiL >= 0 && r.neiL < hd.nT;
                S rwS = S(0), hwf = S(0), kO, kN;
                double Vo = 1.0, Vn = 1.0;
                if constexpr (sizeof(S) == 4) {
                    kO = A.dt * fg.invVo;
                    kN = A.dt * fg.invVn;
                    if (r.w >= 0) {
                        rwS = A.rhoWs[r.w];
                        hwf = A.wall4[r.w].x;
                    }
                } else {
                    kO = kN = S(0);
                    Vo = b.vol[A.cells[hd.cellStart + r.ownL]];
                    Vn = r.neiL >= 0 ? b.vol[A.cells[hd.cellStart + r.neiL]] : 1.0;
                    if (r.w >= 0) {
                        rwS = b.rhoW[r.w];
                        hwf = (b.R * b.Tw[r.w]) * (b.K + 3 - D);
                    }
                }
#pragma unroll
                for (int j = 0; j < NPL; ++j) {
                    const int col = j * 32 + lane, v = v0 + col;
                    const S* xi = dv.xi[j];
                    S xs = S(0);
#pragma unroll
                    for (int q = 0; q < D; ++q) xs += xi[q] * fg.Sv[q];
                    S gf, hf = S(0);
                    if (face_value<S, D, H>(A, r, fg, sg, sh, KC, col, v, xi, xs, gf, hf)) {
                        rf.apply(xi, gf, hf);
                    } else {  // incoming wall DV: rho_w M(U_w, T_w), not relaxed
                        gf = rwS * A.Mw[(size_t)r.w * Vp + v];
                        if (H) hf = gf * hwf;
                    }
                    const S F = xs * gf, Fh = xs * hf;
                    if constexpr (sizeof(S) == 8) {
                        if (ownIn) {
                            sa[r.ownL * KC + col] -= F * b.dt / Vo;
                            if (H) sah[r.ownL * KC + col] -= Fh * b.dt / Vo;
                        }
                        if (neiIn) {
                            sa[r.neiL * KC + col] += F * b.dt / Vn;
                            if (H) sah[r.neiL * KC + col] += Fh * b.dt / Vn;
                        }
                    } else {
                        if (ownIn) {
                            sa[r.ownL * KC + col] -= F * kO;
                            if (H) sah[r.ownL * KC + col] -= Fh * kO;
                        }
                        if (neiIn) {
                            sa[r.neiL * KC + col] += F * kN;
                            if (H) sah[r.neiL * KC + col] += Fh * kN;
                        }
                    }
                }
            }
            __syncthreads();
        }
        for (int lc = warp; lc < hd.nT; lc += NW) {
            const int c = A.cells[hd.cellStart + lc];
            S ur[3];
            if constexpr (sizeof(S) == 4) {
                const float4 u4 = reinterpret_cast<const float4*>(A.cc + (size_t)c * kNCoef)[0];
                ur[0] = u4.x; ur[1] = u4.y; ur[2] = u4.z;
            } else {
                ur[0] = b.U[3 * c]; ur[1] = b.U[3 * c + 1]; ur[2] = b.U[3 * c + 2];
            }
            S m[NS];
#pragma unroll
            for (int s = 0; s < NS; ++s) m[s] = S(0);
#pragma unroll
            for (int j = 0; j < NPL; ++j) {
                const int col = j * 32 + lane, v = v0 + col;
                const S g = sa[lc * KC + col];
                const S h = H ? sah[lc * KC + col] : S(0);
                A.gTn[(size_t)c * Vp + v] = g;
                if (H) A.hTn[(size_t)c * Vp + v] = h;
                S cc[3];
#pragma unroll
                for (int k = 0; k < D; ++k) cc[k] = dv.xi[j][k] - ur[k];
                add_moments<S, D, H, NS, S>(m, dv.w[j], g, h, cc);
            }
            const S tot = reduce_scatter<NS, S>(m, lane);
            if (writer && myslot < SL::NM) mom[lc * NS + myslot].add(tot);
        }
    }
    __syncthreads();
    // ---- finalize cells of T (FP64): macros for the next step
    for (int lc = threadIdx.x; lc < hd.nT; lc += NW * 32) {
        const int c = A.cells[hd.cellStart + lc];
        double M[NS];
        for (int s = 0; s < NS; ++s) M[s] = mom[lc * NS + s].value() * A.invGscale;
        double ur[3];
        if constexpr (sizeof(S) == 4) {
            const float* blk = A.cc + (size_t)c * kNCoef;
            ur[0] = blk[0]; ur[1] = blk[1]; ur[2] = blk[2];
        } else {
            ur[0] = b.U[3 * c]; ur[1] = b.U[3 * c + 1]; ur[2] = b.U[3 * c + 2];
        }
        double rho, U[3], T, tau, qr[3];
        macros_from_moments<D, H>(M, ur, b, rho, U, T, tau, qr);
        const double fac = 2.0 * tau / (2.0 * tau + b.dt * b.Pr);
        double q[3] = {fac * qr[0], fac * qr[1], fac * qr[2]};
        A.rhoN[c] = rho;
        A.TN[c] = T;
        A.tauN[c] = tau;
        for (int k = 0; k < 3; ++k) { A.UN[3 * c + k] = U[k]; A.qN[3 * c + k] = q[k]; }
        if constexpr (sizeof(S) == 4) write_coef<D>(A.ccn + (size_t)c * kNCoef, rho, U, T, q, tau, b, A.gscale);
        if (!(rho > 0.0) || !(T > 0.0) || !isfinite(U[0] + U[1] + U[2] + q[0] + q[1] + q[2])) atomicExch(b.status, 5);
    }
}

// ------------------------------------------------------------ set-up kernels
template <int D>
__global__ void k_cell_coef(StepArgs b, float* cc, double gs) {
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < b.nC; c += gridDim.x * blockDim.x) {
        const double U[3] = {b.U[3 * c], b.U[3 * c + 1], b.U[3 * c + 2]};
        const double q[3] = {b.q[3 * c], b.q[3 * c + 1], b.q[3 * c + 2]};
        write_coef<D>(cc + (size_t)c * kNCoef, b.rho[c], U, b.T[c], q, b.tau[c], b, gs);
    }
}

// Face reference velocities (FP32 path): current face velocity, wall velocity on walls.
static __global__ void k_face_uref(StepArgs b, float4* uref4) {
    for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < b.nA; a += gridDim.x * blockDim.x) {
        // walls: moments about U_w; internal and open boundary faces: the face velocity
        const bool wall = a >= b.nI && b.bKind[a - b.nI] == kBcMaxwell;
        const double* u = wall ? b.Uw + 3 * (a - b.nI) : b.UF + 3 * a;
        uref4[a] = make_float4((float)u[0], (float)u[1], (float)u[2], 0.0f);
    }
}

// Wall Maxwellian per DV (equilibriumMaxwellByRho, discreteVelocity.C:1063-1075)
// and its incoming-half moments about U_w (xi.S <= 0, as updateGHbarSurfMaxwellWallIn).
template <typename S, int D, bool H>
__global__ void k_wall_tables(StepArgs b, S* Mw, double* Min) {
    using SL = Slots<D, H>;
    constexpr int NS = SL::NS;
    __shared__ double red[32 * NS];
    const int w = blockIdx.x;
    const int f = b.nI + w;
    const double* Sf = b.Sf + 3 * f;
    const double Tw = b.Tw[w];
    const double* Uw = b.Uw + 3 * w;
    double m[NS];
    for (int s = 0; s < NS; ++s) m[s] = 0.0;
    for (int v = threadIdx.x; v < b.Vp; v += blockDim.x) {
        const double x0 = b.xi[v], x1 = b.xi[b.Vp + v], x2 = b.xi[2 * b.Vp + v];
        const double M = maxwell_by_rho_ref(Uw[0], Uw[1], Uw[2], Tw, x0, x1, x2, b.R, b.D);
        Mw[(size_t)w * b.Vp + v] = (S)M;
        const double xs = x0 * Sf[0] + x1 * Sf[1] + x2 * Sf[2];
        if (xs <= 0 && v < b.nV) {
            const double c[3] = {x0 - Uw[0], x1 - Uw[1], x2 - Uw[2]};
            const double hh = M * (b.R * Tw) * (b.K + 3 - D);
            add_moments<double, D, H, NS, double>(m, b.w[v], M, hh, c);
        }
    }
    block_sum<NS>(m, red);
    if (threadIdx.x == 0)
        for (int s = 0; s < NS; ++s) Min[(size_t)w * NS + s] = m[s];
}

}  // namespace dugks
