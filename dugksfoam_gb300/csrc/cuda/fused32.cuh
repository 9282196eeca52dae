// FP32 fused sweeps (fast path).  Same two-sweep algorithm as fused_kernels.cuh
// (see fused_impl.cuh for the pass-by-pass mapping to the reference), with
// three changes that matter on GB300:
//
//  * each lane owns NPL consecutive discrete velocities (vector loads and
//    stores of g~ rows; one warp task covers KC = 32*NPL velocities), so the
//    per-face and per-row fixed costs -- metadata loads, the warp
//    reduce-scatter of the moments -- are paid once per KC velocities;
//  * the upwind side is chosen per velocity inside a single stencil loop (both
//    sides' rows are read, one gradient is formed), so warps never run the
//    owner- and neighbour-side reconstructions as divergent paths;
//  * the distributions are stored as deviations from a fixed rest Maxwellian:
//      G = gscale * g - Mref(xi),   Mref = exp(-|xi|^2 / (2 R T0)),
//    gscale = (2 pi R T0)^(D/2) / rho0 (h likewise with Href = Mref R T0 (K+3-D)).
//    Every pass is linear in g, Mref is uniform in space, so the gradient,
//    reconstruction, flux and update act on G unchanged; the relaxations use
//    g = G + Mref; the moments of Mref about any reference velocity are added
//    back exactly in FP64.  Storing the O(0.01-0.1) deviation instead of the
//    O(1) distribution cuts the FP32 storage rounding by the same factor.
//    (The Mref part of the face flux, Mref xi.sum_f(+-S_f), vanishes for a
//    closed cell and is not formed.)
#pragma once

#include "fused_impl.cuh"

namespace dugks {

template <int NPL>
__device__ __forceinline__ void ldv(float (&d)[NPL], const float* p) {
    if constexpr (NPL == 4) {
        const float4 t = *reinterpret_cast<const float4*>(p);
        d[0] = t.x; d[1] = t.y; d[2] = t.z; d[3] = t.w;
    } else if constexpr (NPL == 2) {
        const float2 t = *reinterpret_cast<const float2*>(p);
        d[0] = t.x; d[1] = t.y;
    } else {
        d[0] = *p;
    }
}
template <int NPL>
__device__ __forceinline__ void stv(float* p, const float (&d)[NPL]) {
    if constexpr (NPL == 4) {
        *reinterpret_cast<float4*>(p) = make_float4(d[0], d[1], d[2], d[3]);
    } else if constexpr (NPL == 2) {
        *reinterpret_cast<float2*>(p) = make_float2(d[0], d[1]);
    } else {
        *p = d[0];
    }
}

// Streaming (evict-first) access for the g~ rows: they are touched once per
// sweep, so they should not push the tile's metadata out of L1.
template <int NPL>
__device__ __forceinline__ void ldv_cs(float (&d)[NPL], const float* p) {
    if constexpr (NPL == 4) {
        const float4 t = __ldcs(reinterpret_cast<const float4*>(p));
        d[0] = t.x; d[1] = t.y; d[2] = t.z; d[3] = t.w;
    } else if constexpr (NPL == 2) {
        const float2 t = __ldcs(reinterpret_cast<const float2*>(p));
        d[0] = t.x; d[1] = t.y;
    } else {
        d[0] = __ldcs(p);
    }
}
template <int NPL>
__device__ __forceinline__ void stv_cs(float* p, const float (&d)[NPL]) {
    if constexpr (NPL == 4) {
        __stcs(reinterpret_cast<float4*>(p), make_float4(d[0], d[1], d[2], d[3]));
    } else if constexpr (NPL == 2) {
        __stcs(reinterpret_cast<float2*>(p), make_float2(d[0], d[1]));
    } else {
        __stcs(p, d[0]);
    }
}

// DV constants of this lane's NPL consecutive velocities in the current chunk.
template <int D, int NPL>
struct Lane32 {
    float x[NPL], y[NPL], z[NPL], w[NPL], mr[NPL];
    __device__ __forceinline__ void load(const FusedArgs<float>& A, int v0, int lane) {
        const int Vp = A.b.Vp, v = v0 + lane * NPL;
        ldv<NPL>(x, A.xi + v);
        ldv<NPL>(y, A.xi + Vp + v);
        if (D == 3) ldv<NPL>(z, A.xi + 2 * Vp + v);
        else
#pragma unroll
            for (int j = 0; j < NPL; ++j) z[j] = 0.0f;
        ldv<NPL>(w, A.w + v);
        ldv<NPL>(mr, A.mref + v);
    }
};

// Shakhov relaxation in deviation form: out = G - a (G + Mref) + a g^S.
template <int D, bool H>
struct Eq32 {
    float ux, uy, uz, kexp, invRT, qx, qy, qz, a, aA, RT, KD, K2, hf;
    __device__ __forceinline__ void load(const float* blk, float aw, int K, float hrefFac) {
        const float4 b0 = reinterpret_cast<const float4*>(blk)[0];
        const float4 b1 = reinterpret_cast<const float4*>(blk)[1];
        const float4 b2 = reinterpret_cast<const float4*>(blk)[2];
        ux = b0.x; uy = b0.y; uz = b0.z; kexp = b0.w;
        invRT = b1.x; qx = b1.y; qy = b1.z; qz = b1.w;
        RT = b2.y;
        a = aw;
        aA = aw * b2.x;
        KD = (float)(K + 3 - D);
        K2 = -2.0f * (float)K;
        hf = hrefFac;
    }
    __device__ __forceinline__ float tau(const float* blk) const { return blk[10]; }
    __device__ __forceinline__ void relax(float xx, float xy, float xz, float mr, float& g, float& h) const {
        const float cx = xx - ux, cy = xy - uy;
        const float cz = D == 3 ? xz - uz : 0.0f;
        const float c2 = D == 3 ? fmaf(cz, cz, fmaf(cy, cy, cx * cx)) : fmaf(cy, cy, cx * cx);
        const float e = exp2f(kexp * c2) * aA;
        const float phi = D == 3 ? fmaf(cz, qz, fmaf(cy, qy, cx * qx)) : fmaf(cy, qy, cx * qx);
        const float c2n = c2 * invRT;
        const float ags = fmaf(e * phi, c2n - (float)(D + 2), e);
        g = fmaf(-a, g + mr, g + ags);
        if (H) {
            const float eh = e * RT;
            const float ahs = fmaf(eh * phi, fmaf(c2n - (float)D, KD, K2), eh * KD);
            h = fmaf(-a, h + mr * hf, h + ahs);
        }
    }
};

template <int D, bool H>
__device__ __forceinline__ void eq_cell(Eq32<D, H>& e, const FusedArgs<float>& A, int c) {
    const float* blk = A.cc + (size_t)c * kNCoef;
    e.load(blk, 1.5f * A.dt / (2.0f * blk[10] + A.dt), A.b.K, A.hrefFac);
}
template <int D, bool H>
__device__ __forceinline__ void eq_face(Eq32<D, H>& e, const FusedArgs<float>& A, int a) {
    const float* blk = A.fc + (size_t)a * kNCoef;
    const float hh = 0.5f * A.dt;
    e.load(blk, hh / (2.0f * blk[10] + hh), A.b.K, A.hrefFac);
}

// gbar+ rows of T u H1 u H2 (and for sweep B the g~new partial of T's rows).
// Two rows per warp iteration keep two row loads in flight.
template <int D, bool H, int NPL, bool PART>
__device__ __forceinline__ void row32(const FusedArgs<float>& A, const TileHdr& hd, const Lane32<D, NPL>& L, int lc,
                                      const float (&g0)[NPL], const float (&h0)[NPL], const Eq32<D, H>& eq, int lane,
                                      float* sg, float* sh, float* sa, float* sah) {
    constexpr int KC = 32 * NPL;
    float g[NPL], h[NPL];
#pragma unroll
    for (int j = 0; j < NPL; ++j) {
        g[j] = g0[j];
        h[j] = H ? h0[j] : 0.0f;
        eq.relax(L.x[j], L.y[j], L.z[j], L.mr[j], g[j], h[j]);
    }
    stv<NPL>(sg + lc * KC + lane * NPL, g);
    if (H) stv<NPL>(sh + lc * KC + lane * NPL, h);
    if (PART && lc < hd.nT) {
        float pa[NPL], ph[NPL];
#pragma unroll
        for (int j = 0; j < NPL; ++j) {
            pa[j] = fmaf(g[j] - g0[j], 1.0f / 3.0f, g[j]);
            if (H) ph[j] = fmaf(h[j] - h0[j], 1.0f / 3.0f, h[j]);
        }
        stv<NPL>(sa + lc * KC + lane * NPL, pa);
        if (H) stv<NPL>(sah + lc * KC + lane * NPL, ph);
    }
}

template <int D, bool H, int NPL, int NW, bool PART>
__device__ __forceinline__ void rows32(const FusedArgs<float>& A, const TileHdr& hd, const Lane32<D, NPL>& L, int v0,
                                       int lane, int warp, float* sg, float* sh, float* sa, float* sah) {
    const int Vp = A.b.Vp;
    for (int l0 = warp; l0 < hd.nT2; l0 += 2 * NW) {
        const int l1 = l0 + NW;
        const bool two = l1 < hd.nT2;
        const int c0 = A.cells[hd.cellStart + l0];
        const int c1 = two ? A.cells[hd.cellStart + l1] : c0;
        const size_t i0 = (size_t)c0 * Vp + v0 + lane * NPL, i1 = (size_t)c1 * Vp + v0 + lane * NPL;
        float ga[NPL], ha[NPL], gb[NPL], hb[NPL];
        ldv_cs<NPL>(ga, A.gT + i0);
        ldv_cs<NPL>(gb, A.gT + i1);
        if (H) {
            ldv_cs<NPL>(ha, A.hT + i0);
            ldv_cs<NPL>(hb, A.hT + i1);
        } else {
#pragma unroll
            for (int j = 0; j < NPL; ++j) { ha[j] = 0.0f; hb[j] = 0.0f; }
        }
        Eq32<D, H> e0, e1;
        eq_cell<D, H>(e0, A, c0);
        eq_cell<D, H>(e1, A, c1);
        row32<D, H, NPL, PART>(A, hd, L, l0, ga, ha, e0, lane, sg, sh, sa, sah);
        if (two) row32<D, H, NPL, PART>(A, hd, L, l1, gb, hb, e1, lane, sg, sh, sa, sah);
    }
}

// Face record + geometry in registers.
struct Face32 {
    TileFace r;
    float Sx, Sy, Sz, iVo, dOx, dOy, dOz, iVn, dNx, dNy, dNz;
    __device__ __forceinline__ void load(const FusedArgs<float>& A, int rec) {
        const int4* p = reinterpret_cast<const int4*>(A.faces + rec);
        const int4 a = p[0], b = p[1];
        r.ownL = a.x; r.neiL = a.y; r.a = a.z; r.w = a.w;
        r.stO0 = b.x; r.stO1 = b.y; r.stN0 = b.z; r.stN1 = b.w;
        const float4 g0 = A.fg4[3 * (size_t)rec], g1 = A.fg4[3 * (size_t)rec + 1], g2 = A.fg4[3 * (size_t)rec + 2];
        Sx = g0.x; Sy = g0.y; Sz = g0.z; iVo = g0.w;
        dOx = g1.x; dOy = g1.y; dOz = g1.z; iVn = g1.w;
        dNx = g2.x; dNy = g2.y; dNz = g2.z;
    }
};

// Upwind reconstruction gbar_f = gbar+_u + sum_e (L_e.(d_u - xi dt/2)) (gbar+_o(e) - gbar+_u)
// for this lane's NPL velocities, u = owner (side 0) or neighbour (side 1) per
// velocity; tie (xi.S == 0) velocities average both sides.  For walls only the
// owner side exists.  When GRADW is set the owner gradient itself is also
// returned (lagged boundary gradient of walls).
template <int D, bool H, int NPL, bool WALL>
__device__ __forceinline__ void recon32(const FusedArgs<float>& A, const Face32& F, const Lane32<D, NPL>& L,
                                        const float* sg, const float* sh, int lane, int v0, const float (&xs)[NPL],
                                        float (&gf)[NPL], float (&hf)[NPL], float (&gw)[D][NPL],
                                        float (&hw)[D][NPL]) {
    constexpr int KC = 32 * NPL;
    const float hdt = 0.5f * A.dt;
    const int col = lane * NPL;
    const int Vp = A.b.Vp;
    // side per velocity: 0 owner, 1 neighbour, 2 tie (both)
    int side[NPL];
    bool anyTie = false;
#pragma unroll
    for (int j = 0; j < NPL; ++j) {
        side[j] = WALL ? 0 : (xs[j] > 0.0f ? 0 : (xs[j] < 0.0f ? 1 : 2));
        anyTie |= side[j] == 2;
    }
    float cO[NPL], cN[NPL], hO[NPL], hN[NPL];
    ldv<NPL>(cO, sg + F.r.ownL * KC + col);
    if (H) ldv<NPL>(hO, sh + F.r.ownL * KC + col);
    if (!WALL) {
        ldv<NPL>(cN, sg + F.r.neiL * KC + col);
        if (H) ldv<NPL>(hN, sh + F.r.neiL * KC + col);
    }
    float accG[NPL], accH[NPL], accG2[NPL], accH2[NPL];
#pragma unroll
    for (int j = 0; j < NPL; ++j) {
        accG[j] = 0.0f; accH[j] = 0.0f; accG2[j] = 0.0f; accH2[j] = 0.0f;
        if (WALL) {
#pragma unroll
            for (int k = 0; k < D; ++k) { gw[k][j] = 0.0f; if (H) hw[k][j] = 0.0f; }
        }
    }
    const int nO = F.r.stO1 - F.r.stO0, nN = WALL ? 0 : F.r.stN1 - F.r.stN0;
    const int nE = nO > nN ? nO : nN;
    for (int k = 0; k < nE; ++k) {
        // owner-side entry
        float LOx = 0.f, LOy = 0.f, LOz = 0.f, aO = 0.f;
        float rO[NPL], qO[NPL];
#pragma unroll
        for (int j = 0; j < NPL; ++j) { rO[j] = cO[j]; qO[j] = H ? hO[j] : 0.f; }
        if (k < nO) {
            const float4 e = A.st4[F.r.stO0 + k];
            const int o = __float_as_int(e.w);
            LOx = e.x; LOy = e.y; LOz = e.z;
            aO = fmaf(LOy, F.dOy, LOx * F.dOx);
            if (D == 3) aO = fmaf(LOz, F.dOz, aO);
            if (o >= 0) {
                ldv<NPL>(rO, sg + o * KC + col);
                if (H) ldv<NPL>(qO, sh + o * KC + col);
            } else {
                const int wf = -o - 1;
                const float idc = A.wall4[wf].y;
                float tg[NPL], th[NPL];
                ldv<NPL>(tg, A.Gbg + (size_t)wf * Vp + v0 + col);
                if (H) ldv<NPL>(th, A.Gbh + (size_t)wf * Vp + v0 + col);
#pragma unroll
                for (int j = 0; j < NPL; ++j) {
                    rO[j] = fmaf(tg[j], idc, cO[j]);
                    if (H) qO[j] = fmaf(th[j], idc, hO[j]);
                }
            }
        }
        float LNx = 0.f, LNy = 0.f, LNz = 0.f, aN = 0.f;
        float rN[NPL], qN[NPL];
        if (!WALL) {
#pragma unroll
            for (int j = 0; j < NPL; ++j) { rN[j] = cN[j]; qN[j] = H ? hN[j] : 0.f; }
            if (k < nN) {
                const float4 e = A.st4[F.r.stN0 + k];
                const int o = __float_as_int(e.w);
                LNx = e.x; LNy = e.y; LNz = e.z;
                aN = fmaf(LNy, F.dNy, LNx * F.dNx);
                if (D == 3) aN = fmaf(LNz, F.dNz, aN);
                if (o >= 0) {
                    ldv<NPL>(rN, sg + o * KC + col);
                    if (H) ldv<NPL>(qN, sh + o * KC + col);
                } else {
                    const int wf = -o - 1;
                    const float idc = A.wall4[wf].y;
                    float tg[NPL], th[NPL];
                    ldv<NPL>(tg, A.Gbg + (size_t)wf * Vp + v0 + col);
                    if (H) ldv<NPL>(th, A.Gbh + (size_t)wf * Vp + v0 + col);
#pragma unroll
                    for (int j = 0; j < NPL; ++j) {
                        rN[j] = fmaf(tg[j], idc, cN[j]);
                        if (H) qN[j] = fmaf(th[j], idc, hN[j]);
                    }
                }
            }
        }
#pragma unroll
        for (int j = 0; j < NPL; ++j) {
            if (WALL) {
                const float dg = rO[j] - cO[j], dh = H ? qO[j] - hO[j] : 0.f;
                gw[0][j] = fmaf(LOx, dg, gw[0][j]);
                gw[1][j] = fmaf(LOy, dg, gw[1][j]);
                if (D == 3) gw[2][j] = fmaf(LOz, dg, gw[2][j]);
                if (H) {
                    hw[0][j] = fmaf(LOx, dh, hw[0][j]);
                    hw[1][j] = fmaf(LOy, dh, hw[1][j]);
                    if (D == 3) hw[2][j] = fmaf(LOz, dh, hw[2][j]);
                }
                float lx = LOx * L.x[j];
                lx = fmaf(LOy, L.y[j], lx);
                if (D == 3) lx = fmaf(LOz, L.z[j], lx);
                const float beta = fmaf(-hdt, lx, aO);
                accG[j] = fmaf(beta, dg, accG[j]);
                if (H) accH[j] = fmaf(beta, dh, accH[j]);
            } else {
                const bool n = side[j] == 1;
                const float Lx = n ? LNx : LOx, Ly = n ? LNy : LOy, Lz = n ? LNz : LOz, al = n ? aN : aO;
                const float dg = n ? rN[j] - cN[j] : rO[j] - cO[j];
                const float dh = H ? (n ? qN[j] - hN[j] : qO[j] - hO[j]) : 0.f;
                float lx = Lx * L.x[j];
                lx = fmaf(Ly, L.y[j], lx);
                if (D == 3) lx = fmaf(Lz, L.z[j], lx);
                const float beta = fmaf(-hdt, lx, al);
                accG[j] = fmaf(beta, dg, accG[j]);
                if (H) accH[j] = fmaf(beta, dh, accH[j]);
                if (anyTie && side[j] == 2) {  // tie: the neighbour side separately
                    float ln = LNx * L.x[j];
                    ln = fmaf(LNy, L.y[j], ln);
                    if (D == 3) ln = fmaf(LNz, L.z[j], ln);
                    const float bn = fmaf(-hdt, ln, aN);
                    accG2[j] = fmaf(bn, rN[j] - cN[j], accG2[j]);
                    if (H) accH2[j] = fmaf(bn, qN[j] - hN[j], accH2[j]);
                }
            }
        }
    }
#pragma unroll
    for (int j = 0; j < NPL; ++j) {
        if (WALL || side[j] == 0) {
            gf[j] = cO[j] + accG[j];
            if (H) hf[j] = hO[j] + accH[j];
        } else if (side[j] == 1) {
            gf[j] = cN[j] + accG[j];
            if (H) hf[j] = hN[j] + accH[j];
        } else {
            gf[j] = 0.5f * ((cN[j] + accG2[j]) + (cO[j] + accG[j]));
            if (H) hf[j] = 0.5f * ((hN[j] + accH2[j]) + (hO[j] + accH[j]));
        }
    }
}

// Deviation moments of NPL velocities about ur into the lane's slots.
template <int D, bool H, int NPL, int NS>
__device__ __forceinline__ void mom32(float (&m)[NS], const Lane32<D, NPL>& L, const float* ur, const float (&g)[NPL],
                                      const float (&h)[NPL], const bool* use) {
    using SL = Slots<D, H>;
#pragma unroll
    for (int j = 0; j < NPL; ++j) {
        if (use && !use[j]) continue;
        const float c[3] = {L.x[j] - ur[0], L.y[j] - ur[1], D == 3 ? L.z[j] - ur[2] : 0.0f};
        const float wg = L.w[j] * g[j];
        m[0] += wg;
        float c2 = c[0] * c[0];
#pragma unroll
        for (int i = 1; i < D; ++i) c2 = fmaf(c[i], c[i], c2);
#pragma unroll
        for (int i = 0; i < D; ++i) {
            const float t = wg * c[i];
            m[SL::M1 + i] += t;
#pragma unroll
            for (int k = i; k < D; ++k) m[SL::M2 + sym<D>(i, k)] = fmaf(t, c[k], m[SL::M2 + sym<D>(i, k)]);
            m[SL::M3 + i] = fmaf(t, c2, m[SL::M3 + i]);
        }
        if (H) {
            const float wh = L.w[j] * h[j];
            m[SL::H0] += wh;
#pragma unroll
            for (int i = 0; i < D; ++i) m[SL::H1 + i] = fmaf(wh, c[i], m[SL::H1 + i]);
        }
    }
}

// Moments of the reference Maxwellian about u (FP64, scaled units) from its raw
// moments R (slots as Slots<D,H>, taken about the origin).
template <int D, bool H>
__device__ __forceinline__ void ref_moments_about(const double* R, const double* u, double* M) {
    using SL = Slots<D, H>;
    const double r0 = R[0];
    double tr = 0, r1u = 0, uu = 0;
    for (int i = 0; i < D; ++i) {
        tr += R[SL::M2 + sym<D>(i, i)];
        r1u += R[SL::M1 + i] * u[i];
        uu += u[i] * u[i];
    }
    M[0] = r0;
    for (int i = 0; i < D; ++i) {
        M[SL::M1 + i] = R[SL::M1 + i] - u[i] * r0;
        for (int k = i; k < D; ++k)
            M[SL::M2 + sym<D>(i, k)] = R[SL::M2 + sym<D>(i, k)] - u[i] * R[SL::M1 + k] - u[k] * R[SL::M1 + i] + u[i] * u[k] * r0;
        double r2u = 0;
        for (int k = 0; k < D; ++k) r2u += R[SL::M2 + (i <= k ? sym<D>(i, k) : sym<D>(k, i))] * u[k];
        M[SL::M3 + i] = R[SL::M3 + i] - 2.0 * r2u + R[SL::M1 + i] * uu - u[i] * tr + 2.0 * u[i] * r1u - u[i] * uu * r0;
    }
    if (H) {
        M[SL::H0] = R[SL::H0];
        for (int i = 0; i < D; ++i) M[SL::H1 + i] = R[SL::H1 + i] - u[i] * R[SL::H0];
    }
}

// ---------------------------------------------------------------- sweep A
template <int D, bool H, int NPL, int NW>
__global__ void __launch_bounds__(NW * 32, 1) k_sweep_face32(FusedArgs<float> A) {
    using SL = Slots<D, H>;
    constexpr int NS = SL::NS, KC = 32 * NPL;
    extern __shared__ __align__(16) unsigned char smem[];
    const TileHdr hd = A.hdr[blockIdx.x];
    const StepArgs& b = A.b;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int Vp = b.Vp;
    const size_t rowBytes = (size_t)hd.nT2 * KC * sizeof(float) * (H ? 2 : 1);
    float* sg = reinterpret_cast<float*>(smem);
    float* sh = sg + (size_t)hd.nT2 * KC;
    Acc<float>* mom = reinterpret_cast<Acc<float>*>(smem + ((rowBytes + 15) & ~size_t(15)));
    for (int i = threadIdx.x; i < hd.nFA * NS; i += NW * 32) mom[i].zero();
    const int nChunks = Vp / KC;
    const int myslot = slot_of<NS>(lane);
    const bool writer = NS == 16 ? (lane & 1) == 0 : true;

    for (int ch = 0; ch < nChunks; ++ch) {
        const int v0 = ch * KC;
        Lane32<D, NPL> L;
        L.load(A, v0, lane);
        __syncthreads();
        rows32<D, H, NPL, NW, false>(A, hd, L, v0, lane, warp, sg, sh, nullptr, nullptr);
        __syncthreads();
        for (int lf = warp; lf < hd.nFA; lf += NW) {
            Face32 F;
            F.load(A, hd.faceStart + lf);
            const float4 u4 = A.uref4[F.r.a];
            const float ur[3] = {u4.x, u4.y, u4.z};
            float xs[NPL];
#pragma unroll
            for (int j = 0; j < NPL; ++j) {
                xs[j] = fmaf(L.y[j], F.Sy, L.x[j] * F.Sx);
                if (D == 3) xs[j] = fmaf(L.z[j], F.Sz, xs[j]);
            }
            float gf[NPL], hf[NPL], gw[D][NPL], hw[D][NPL];
            float m[NS];
#pragma unroll
            for (int s = 0; s < NS; ++s) m[s] = 0.0f;
            if (F.r.w >= 0) {
                recon32<D, H, NPL, true>(A, F, L, sg, sh, lane, v0, xs, gf, hf, gw, hw);
                float gn[NPL], hn[NPL];
                bool use[NPL];
#pragma unroll
                for (int j = 0; j < NPL; ++j) {
                    gn[j] = gw[0][j] * F.dNx;
                    gn[j] = fmaf(gw[1][j], F.dNy, gn[j]);
                    if (D == 3) gn[j] = fmaf(gw[2][j], F.dNz, gn[j]);
                    if (H) {
                        hn[j] = hw[0][j] * F.dNx;
                        hn[j] = fmaf(hw[1][j], F.dNy, hn[j]);
                        if (D == 3) hn[j] = fmaf(hw[2][j], F.dNz, hn[j]);
                    }
                    use[j] = xs[j] > 0.0f;
                    if (use[j]) m[SL::FLUX] = fmaf(L.w[j] * xs[j], gf[j], m[SL::FLUX]);
                }
                const size_t wi = (size_t)F.r.w * Vp + v0 + lane * NPL;
                stv<NPL>(A.Gbgn + wi, gn);
                if (H) stv<NPL>(A.Gbhn + wi, hn);
                mom32<D, H, NPL, NS>(m, L, ur, gf, hf, use);
            } else {
                recon32<D, H, NPL, false>(A, F, L, sg, sh, lane, v0, xs, gf, hf, gw, hw);
                mom32<D, H, NPL, NS>(m, L, ur, gf, hf, nullptr);
            }
            const float tot = reduce_scatter<NS, float>(m, lane);
            if (writer && myslot <= SL::FLUX) mom[lf * NS + myslot].add(tot);
        }
    }
    __syncthreads();
    // ---- finalize owned faces (FP64)
    for (int lf = threadIdx.x; lf < hd.nFA; lf += NW * 32) {
        const TileFace r = A.faces[hd.faceStart + lf];
        const float4 u4 = A.uref4[r.a];
        const double ur[3] = {u4.x, u4.y, u4.z};
        double M[NS], Rm[NS];
        for (int s = 0; s < NS; ++s) M[s] = mom[lf * NS + s].value();
        double rw = 0.0;
        if (r.w >= 0) {  // outgoing: deviation + reference parts; incoming: rho_w * Mw
            const double* RO = A.wallRefOut + (size_t)r.w * NS;
            for (int s = 0; s <= SL::FLUX; ++s) M[s] += RO[s];
            rw = M[SL::FLUX] / b.incAbs[r.w];
            for (int s = 0; s < SL::NM; ++s) M[s] += rw * A.Min[(size_t)r.w * NS + s];
        } else {
            ref_moments_about<D, H>(A.refMom, ur, Rm);
            for (int s = 0; s < SL::NM; ++s) M[s] += Rm[s];
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
        write_coef<D>(A.fc + (size_t)a * kNCoef, rho, U, T, q, tau, b, A.gscale);
        if (r.w < 0) A.uref4[a] = make_float4((float)U[0], (float)U[1], (float)U[2], 0.0f);
        if (r.w >= 0) {
            const int w = r.w;
            b.rhoW[w] = rw * A.invGscale;
            A.rhoWs[w] = (float)rw;
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
template <int D, bool H, int NPL, int NW>
__global__ void __launch_bounds__(NW * 32, 1) k_sweep_cell32(FusedArgs<float> A) {
    using SL = Slots<D, H>;
    constexpr int NS = SL::NS, KC = 32 * NPL;
    extern __shared__ __align__(16) unsigned char smem[];
    const TileHdr hd = A.hdr[blockIdx.x];
    const StepArgs& b = A.b;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int Vp = b.Vp;
    const size_t rb2 = ((size_t)hd.nT2 * KC * sizeof(float) * (H ? 2 : 1) + 15) & ~size_t(15);
    const size_t rb1 = ((size_t)hd.nT * KC * sizeof(float) * (H ? 2 : 1) + 15) & ~size_t(15);
    float* sg = reinterpret_cast<float*>(smem);
    float* sh = sg + (size_t)hd.nT2 * KC;
    float* sa = reinterpret_cast<float*>(smem + rb2);
    float* sah = sa + (size_t)hd.nT * KC;
    Acc<float>* mom = reinterpret_cast<Acc<float>*>(smem + rb2 + rb1);
    for (int i = threadIdx.x; i < hd.nT * NS; i += NW * 32) mom[i].zero();
    const int nChunks = Vp / KC;
    const int myslot = slot_of<NS>(lane);
    const bool writer = NS == 16 ? (lane & 1) == 0 : true;
    const int col = lane * NPL;

    for (int ch = 0; ch < nChunks; ++ch) {
        const int v0 = ch * KC;
        Lane32<D, NPL> L;
        L.load(A, v0, lane);
        __syncthreads();
        rows32<D, H, NPL, NW, true>(A, hd, L, v0, lane, warp, sg, sh, sa, sah);
        __syncthreads();
        for (int ci = 0; ci < hd.nColors; ++ci) {
            const int k0 = A.colorOff[hd.colStart + ci], k1 = A.colorOff[hd.colStart + ci + 1];
            for (int k = k0 + warp; k < k1; k += NW) {
                const int lf = A.colorPerm[hd.permStart + k];
                Face32 F;
                F.load(A, hd.faceStart + lf);
                Eq32<D, H> eq;
                eq_face<D, H>(eq, A, F.r.a);
                float xs[NPL];
#pragma unroll
                for (int j = 0; j < NPL; ++j) {
                    xs[j] = fmaf(L.y[j], F.Sy, L.x[j] * F.Sx);
                    if (D == 3) xs[j] = fmaf(L.z[j], F.Sz, xs[j]);
                }
                float gf[NPL], hf[NPL], gw[D][NPL], hw[D][NPL];
                if (F.r.w >= 0) {
                    recon32<D, H, NPL, true>(A, F, L, sg, sh, lane, v0, xs, gf, hf, gw, hw);
                    const float rws = A.rhoWs[F.r.w], hwf = A.wall4[F.r.w].x;
                    float mw[NPL];
                    ldv<NPL>(mw, A.Mw + (size_t)F.r.w * Vp + v0 + col);
#pragma unroll
                    for (int j = 0; j < NPL; ++j) {
                        if (xs[j] > 0.0f) {
                            eq.relax(L.x[j], L.y[j], L.z[j], L.mr[j], gf[j], hf[j]);
                        } else {  // incoming: rho_w Mw (deviation), not relaxed
                            const float gi = rws * mw[j];
                            gf[j] = gi - L.mr[j];
                            if (H) hf[j] = gi * hwf - L.mr[j] * A.hrefFac;
                        }
                    }
                } else {
                    recon32<D, H, NPL, false>(A, F, L, sg, sh, lane, v0, xs, gf, hf, gw, hw);
#pragma unroll
                    for (int j = 0; j < NPL; ++j) eq.relax(L.x[j], L.y[j], L.z[j], L.mr[j], gf[j], hf[j]);
                }
                const bool ownIn = F.r.ownL < hd.nT, neiIn = F.r.neiL >= 0 && F.r.neiL < hd.nT;
                const float kO = A.dt * F.iVo, kN = A.dt * F.iVn;
                if (ownIn) {
                    float t[NPL], th[NPL];
                    ldv<NPL>(t, sa + F.r.ownL * KC + col);
                    if (H) ldv<NPL>(th, sah + F.r.ownL * KC + col);
#pragma unroll
                    for (int j = 0; j < NPL; ++j) {
                        t[j] = fmaf(-xs[j] * kO, gf[j], t[j]);
                        if (H) th[j] = fmaf(-xs[j] * kO, hf[j], th[j]);
                    }
                    stv<NPL>(sa + F.r.ownL * KC + col, t);
                    if (H) stv<NPL>(sah + F.r.ownL * KC + col, th);
                }
                if (neiIn) {
                    float t[NPL], th[NPL];
                    ldv<NPL>(t, sa + F.r.neiL * KC + col);
                    if (H) ldv<NPL>(th, sah + F.r.neiL * KC + col);
#pragma unroll
                    for (int j = 0; j < NPL; ++j) {
                        t[j] = fmaf(xs[j] * kN, gf[j], t[j]);
                        if (H) th[j] = fmaf(xs[j] * kN, hf[j], th[j]);
                    }
                    stv<NPL>(sa + F.r.neiL * KC + col, t);
                    if (H) stv<NPL>(sah + F.r.neiL * KC + col, th);
                }
            }
            __syncthreads();
        }
        for (int lc = warp; lc < hd.nT; lc += NW) {
            const int c = A.cells[hd.cellStart + lc];
            const float4 u4 = reinterpret_cast<const float4*>(A.cc + (size_t)c * kNCoef)[0];
            const float ur[3] = {u4.x, u4.y, u4.z};
            float g[NPL], h[NPL];
            ldv<NPL>(g, sa + lc * KC + col);
            if (H) ldv<NPL>(h, sah + lc * KC + col);
            else
#pragma unroll
                for (int j = 0; j < NPL; ++j) h[j] = 0.0f;
            const size_t gi = (size_t)c * Vp + v0 + col;
            stv_cs<NPL>(A.gTn + gi, g);
            if (H) stv_cs<NPL>(A.hTn + gi, h);
            float m[NS];
#pragma unroll
            for (int s = 0; s < NS; ++s) m[s] = 0.0f;
            mom32<D, H, NPL, NS>(m, L, ur, g, h, nullptr);
            const float tot = reduce_scatter<NS, float>(m, lane);
            if (writer && myslot < SL::NM) mom[lc * NS + myslot].add(tot);
        }
    }
    __syncthreads();
    // ---- finalize cells of T (FP64)
    for (int lc = threadIdx.x; lc < hd.nT; lc += NW * 32) {
        const int c = A.cells[hd.cellStart + lc];
        const float* blk = A.cc + (size_t)c * kNCoef;
        const double ur[3] = {blk[0], blk[1], blk[2]};
        double M[NS], Rm[NS];
        for (int s = 0; s < NS; ++s) M[s] = mom[lc * NS + s].value();
        ref_moments_about<D, H>(A.refMom, ur, Rm);
        for (int s = 0; s < SL::NM; ++s) M[s] = (M[s] + Rm[s]) * A.invGscale;
        double rho, U[3], T, tau, qr[3];
        macros_from_moments<D, H>(M, ur, b, rho, U, T, tau, qr);
        const double fac = 2.0 * tau / (2.0 * tau + b.dt * b.Pr);
        double q[3] = {fac * qr[0], fac * qr[1], fac * qr[2]};
        A.rhoN[c] = rho;
        A.TN[c] = T;
        A.tauN[c] = tau;
        for (int k = 0; k < 3; ++k) { A.UN[3 * c + k] = U[k]; A.qN[3 * c + k] = q[k]; }
        write_coef<D>(A.ccn + (size_t)c * kNCoef, rho, U, T, q, tau, b, A.gscale);
        if (!(rho > 0.0) || !(T > 0.0) || !isfinite(U[0] + U[1] + U[2] + q[0] + q[1] + q[2])) atomicExch(b.status, 5);
    }
}

// ------------------------------------------------------------ set-up kernels
// Reference Maxwellian per DV (scaled: exp(-|xi|^2/(2 R T0))), its raw moments
// (scaled, about the origin) and, per wall face, the reference moments over
// the outgoing velocities about U_w plus the reference outgoing flux.
template <int D, bool H>
__global__ void k_ref_tables(StepArgs b, double T0, double hrefFac, float* mref, double* refMom, double* wallRefOut) {
    using SL = Slots<D, H>;
    constexpr int NS = SL::NS;
    __shared__ double red[32 * NS];
    const int blk = blockIdx.x;  // 0: raw moments; 1 + w: wall face w
    double m[NS];
    for (int s = 0; s < NS; ++s) m[s] = 0.0;
    const double* Uw = blk > 0 ? b.Uw + 3 * (blk - 1) : nullptr;
    const double* Sf = blk > 0 ? b.Sf + 3 * (b.nI + blk - 1) : nullptr;
    for (int v = threadIdx.x; v < b.Vp; v += blockDim.x) {
        const double x0 = b.xi[v], x1 = b.xi[b.Vp + v], x2 = b.xi[2 * b.Vp + v];
        const double M = exp(-(x0 * x0 + x1 * x1 + x2 * x2) / (2.0 * b.R * T0));
        if (blk == 0) mref[v] = (float)M;
        const double Mf = (double)(float)M;  // moments of the FP32 value actually subtracted
        const double wv = b.w[v];
        if (blk == 0) {
            const double c[3] = {x0, x1, x2};
            add_moments<double, D, H, NS, double>(m, wv, Mf, Mf * hrefFac, c);
        } else {
            const double xs = x0 * Sf[0] + x1 * Sf[1] + x2 * Sf[2];
            if (xs > 0 && v < b.nV) {
                const double c[3] = {x0 - Uw[0], x1 - Uw[1], x2 - Uw[2]};
                add_moments<double, D, H, NS, double>(m, wv, Mf, Mf * hrefFac, c);
                m[SL::FLUX] += wv * xs * Mf;
            }
        }
    }
    block_sum<NS>(m, red);
    if (threadIdx.x == 0) {
        double* out = blk == 0 ? refMom : wallRefOut + (size_t)(blk - 1) * NS;
        for (int s = 0; s < NS; ++s) out[s] = m[s];
    }
}

// Deviation-form state from FP64 values: G = gscale g - Mref, H = gscale h - Href.
__global__ static void k_init_dev32(StepArgs b, const float* mref, double gs, double hrefFac, float* gT, float* hT) {
    const long long n = (long long)b.nC * b.Vp;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(i / b.Vp), v = (int)(i - (long long)c * b.Vp);
        double ge, he;
        shakhov_ref(b.rho[c], b.U[3 * c], b.U[3 * c + 1], b.U[3 * c + 2], b.T[c], 0.0, 0.0, 0.0, b.xi[v],
                    b.xi[b.Vp + v], b.xi[2 * b.Vp + v], b.R, b.Pr, b.D, b.K, ge, he);
        const double mr = mref[v];
        gT[i] = (float)(ge * gs - mr);
        if (b.hasH) hT[i] = (float)(he * gs - mr * hrefFac);
        if (v == 0) b.tau[c] = tau_ref(b.T[c], b.rho[c], b.muRef, b.omega, b.Tref, b.R);
    }
}

__global__ static void k_export_dev32(StepArgs b, const float* src, const float* mref, double fac, double inv, double* dst) {
    const long long n = (long long)b.nC * b.nV;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(i / b.nV), v = (int)(i - (long long)c * b.nV);
        dst[i] = ((double)src[(long long)c * b.Vp + v] + (double)mref[v] * fac) * inv;
    }
}

__global__ static void k_import_dev32(StepArgs b, const double* src, const float* mref, double fac, double gs, float* dst) {
    const long long n = (long long)b.nC * b.nV;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(i / b.nV), v = (int)(i - (long long)c * b.nV);
        dst[(long long)c * b.Vp + v] = (float)(src[i] * gs - (double)mref[v] * fac);
    }
}

}  // namespace dugks
