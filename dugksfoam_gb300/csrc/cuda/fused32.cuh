// FP32 step (fast path): three launches per step.
//
//  k_face_sides32  (tiles of cells T with a one-ring halo H1, DV chunks of
//                   KC = 32*NPL velocities): gbar+ rows of T u H1 (P1), the
//                   least-squares gradient of each T cell (P2) and the upwind
//                   reconstruction of every face side whose cell is in T (P3),
//                   lagged wall gradients, stored face values and per-side
//                   face moments;
//  k_face_macros32 (one thread per face): Maxwell-wall density (P4), incoming
//                   wall moments (P5), face macros and equilibrium tables (P6);
//  k_cell_gather32 (one warp per cell): face relaxation (P7), flux sum and
//                   g~ update (P8), cell moments and macros (P9).
//
// Layout and arithmetic choices:
//  * each lane owns NPL consecutive discrete velocities held as NPL/2 packed
//    float2 pairs (f32x2 FMA/ADD/MUL), so every per-velocity operation is one
//    packed instruction per pair and the per-face fixed costs (metadata, the
//    warp reduce-scatter of the moments) are paid once per KC velocities;
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
//  * no FP64 instruction runs inside the DV chunk loops (GB300 issues FP64 at
//    1/64 of the FP32 rate): the face sweep's per-chunk warp totals go into
//    FP32 Kahan pairs per face side; the gather keeps per-lane FP32 partial
//    sums over all chunks of a cell and reduces them across the warp once;
//    both are finished in FP64, batched so that whole warps do the FP64 work.
#pragma once

#include "fused_impl.cuh"

namespace dugks {


// 2^x by the hardware approximation (ex2.approx.ftz.f32, PTX ISA).  Flushing
// a result below 2^-126 to zero moves an equilibrium value by less than 1e-38
// of its peak (the grids here reach |xi - U|^2 / 2RT = 48 at T = T0).
__device__ __forceinline__ float ex2f(float x) {
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// Packed FP32 pair arithmetic (sm_100+): each lane's NPL velocities are held
// as NPL/2 float2 pairs and every per-velocity operation is one packed
// instruction per pair.
__device__ __forceinline__ float2 f2(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __ffma2_rn(b, make_float2(-1.0f, -1.0f), a); }
__device__ __forceinline__ float2 sel2(bool x0, bool x1, float2 a, float2 b) {  // per element: x ? a : b
    return make_float2(x0 ? a.x : b.x, x1 ? a.y : b.y);
}

template <int NP>
__device__ __forceinline__ void ldp(float2 (&d)[NP], const float* p) {
    if constexpr (NP == 2) {
        const float4 t = *reinterpret_cast<const float4*>(p);
        d[0] = make_float2(t.x, t.y);
        d[1] = make_float2(t.z, t.w);
    } else {
        d[0] = *reinterpret_cast<const float2*>(p);
    }
}
template <int NP>
__device__ __forceinline__ void stp(float* p, const float2 (&d)[NP]) {
    if constexpr (NP == 2) *reinterpret_cast<float4*>(p) = make_float4(d[0].x, d[0].y, d[1].x, d[1].y);
    else *reinterpret_cast<float2*>(p) = d[0];
}
// Streaming (evict-first) store of the g~new rows: written once, read next step.
template <int NP>
__device__ __forceinline__ void stp_cs(float* p, const float2 (&d)[NP]) {
    if constexpr (NP == 2) __stcs(reinterpret_cast<float4*>(p), make_float4(d[0].x, d[0].y, d[1].x, d[1].y));
    else __stcs(reinterpret_cast<float2*>(p), d[0]);
}

// Per-tile metadata block (int4 units), staged into shared memory once per tile:
//   [nFB][5]  face record {ownL, neiL, a, w} {stO0, stO1, stN0, stN1} (stencil
//             ranges relative to the tile's first entry) and geometry
//             {S, 1/Vo} {dO, 1/Vn} {dN or wall normal}
//   [nEnt]    stencil entries {Lx, Ly, Lz, other}
//   cells (nT2), first stencil entry of each cell of T (nT + 1), as ints
//   padded to whole int4.
__host__ __device__ constexpr int tile_meta32_bound(int nFB, int nEnt, int nT2) {
    return 5 * nFB + nEnt + (nT2 + 3) / 4 + (nT2 + 4) / 4;
}

// Shared memory of the face-sides sweep (all offsets multiples of 16 bytes):
//   2 x rows(T u H1) | face moments | metadata | face Uref | cell equilibria
// (the next DV chunk's raw rows stream into the second row buffer).
// (GR: gradients of the cells of T kept per chunk, [nT][D][g, h][KC], after the rows.)
// With per-cell gradients (GR) the faces read only the rows of T, so the
// halo rows have a single buffer (refilled after the gradient pass) and only
// the rows of T are double-buffered: [T rows x2 | halo rows].
template <int D, bool H, int NPL, bool GR = false>
struct SmemLayout32 {
    static constexpr int KC = 32 * NPL, NS = Slots<D, H>::NS;
    __host__ __device__ static size_t rows(int n) { return (size_t)n * KC * sizeof(float) * (H ? 2 : 1); }
    __host__ __device__ static size_t grad(int nT) { return GR ? (size_t)nT * D * rows(1) : 0; }
    __host__ __device__ static size_t rowBlock(int nRows, int nT) { return GR ? rows(nT) + rows(nRows) : 2 * rows(nRows); }
    __host__ __device__ static size_t mom(int nRows, int nT) { return rowBlock(nRows, nT) + grad(nT); }
    __host__ __device__ static size_t meta(int nRows, int nF, int nT) {
        return mom(nRows, nT) + (size_t)nF * NS * sizeof(Acc<float>);
    }
    static size_t sides(const TileDims& d) {
        return meta(d.nT2, d.nFB, d.nT) + 16 * (size_t)tile_meta32_bound(d.nFB, d.nEnt, d.nT2) + 16 * (size_t)d.nFB +
               48 * (size_t)d.nT2;
    }
};

struct TileMeta32 {
    const int4* F;    // face records [nFB][5]
    const float4* E;  // stencil entries
    const int* C;     // local -> global cell
    const int* S;     // first stencil entry of each cell of T [nT+1]
    float4* dyn;      // per-step tables after the block
};

// Copy the tile's block into shared memory (caller synchronises).
template <int NT>
__device__ __forceinline__ TileMeta32 stage_meta(const FusedArgs<float>& A, const TileHdr& hd, int tile,
                                                 unsigned char* at) {
    int4* sm = reinterpret_cast<int4*>(at);
    const int o0 = A.metaOff[tile], n16 = A.metaOff[tile + 1] - o0;
    const int4* gm = A.meta + o0;
    for (int i = threadIdx.x; i < n16; i += NT) sm[i] = __ldg(gm + i);
    TileMeta32 m;
    m.F = sm;
    m.E = reinterpret_cast<const float4*>(sm + 5 * hd.nFB);
    m.C = reinterpret_cast<const int*>(sm + 5 * hd.nFB + hd.nEnt);
    m.S = reinterpret_cast<const int*>(sm + 5 * hd.nFB + hd.nEnt + (hd.nT2 + 3) / 4);
    m.dyn = reinterpret_cast<float4*>(sm + tile_meta32_bound(hd.nFB, hd.nEnt, hd.nT2));
    return m;
}

#if defined(DUGKS_CHECKED) && DUGKS_CHECKED
// Checked build: every index of a staged tile block within its range (rows
// of T u H1, faces, walls, stencil entries, cells); an index outside is
// replaced by 0 in the staged copy and reported (chk).
template <int NT>
__device__ void check_tile_meta32(const FusedArgs<float>& A, const TileHdr& hd, unsigned char* at) {
    int4* sm = reinterpret_cast<int4*>(at);
    int* st = A.b.status;
    for (int k = threadIdx.x; k < hd.nFB; k += NT) {
        int4& r = sm[5 * k];  // {ownL, neiL, a, w}
        r.x = chk(r.x, hd.nT2, st);
        if (r.y >= 0) r.y = chk(r.y, hd.nT2, st);
        r.z = chk(r.z, A.b.nA, st);
        if (r.w >= 0) r.w = chk(r.w, A.b.nW, st);
        int4& e = sm[5 * k + 1];  // stencil ranges, tile-relative
        e.x = chk(e.x, hd.nEnt + 1, st); e.y = chk(e.y, hd.nEnt + 1, st);
        e.z = chk(e.z, hd.nEnt + 1, st); e.w = chk(e.w, hd.nEnt + 1, st);
    }
    float4* E = reinterpret_cast<float4*>(sm + 5 * hd.nFB);
    for (int k = threadIdx.x; k < hd.nEnt; k += NT) {
        const int o = __float_as_int(E[k].w);
        const int ok = o >= 0 ? chk(o, hd.nT2, st) : -1 - chk(-o - 1, A.b.nW, st);
        E[k].w = __int_as_float(ok);
    }
    int* C = reinterpret_cast<int*>(sm + 5 * hd.nFB + hd.nEnt);
    for (int k = threadIdx.x; k < hd.nT2; k += NT) C[k] = chk(C[k], A.b.nC, st);
    int* S = reinterpret_cast<int*>(sm + 5 * hd.nFB + hd.nEnt + (hd.nT2 + 3) / 4);
    for (int k = threadIdx.x; k <= hd.nT; k += NT) S[k] = chk(S[k], hd.nEnt + 1, st);
}
#endif

// Equilibrium table entry {U, kexp} {1/RT, q'} {a, a A, RT, 0} from a
// coefficient block and the relaxation weight a.
__device__ __forceinline__ void eq_table(float4* q, const float* blk, float a) {
    const float4* b = reinterpret_cast<const float4*>(blk);
    const float4 b2 = b[2];
    q[0] = b[0];
    q[1] = b[1];
    q[2] = make_float4(a, a * b2.x, b2.y, 0.0f);
}
// cell weight 1.5dt/(2tau+dt), face weight h/(2tau+h) with h = dt/2
__device__ __forceinline__ float cell_weight(float dt, const float* blk) { return 1.5f * dt / (2.0f * blk[10] + dt); }
__device__ __forceinline__ float face_weight(float dt, const float* blk) {
    const float hh = 0.5f * dt;
    return hh / (2.0f * blk[10] + hh);
}

// DV constants of this lane's NPL consecutive velocities in the current chunk.
template <int D, int NPL>
struct Lane32 {
    static constexpr int NP = NPL / 2;
    float2 x[NP], y[NP], z[NP], w[NP], mr[NP];
    __device__ __forceinline__ void load(const FusedArgs<float>& A, int v0, int lane) {
        const int Vp = A.b.Vp, v = v0 + lane * NPL;
        ldp<NP>(x, A.xi + v);
        ldp<NP>(y, A.xi + Vp + v);
        if (D == 3) ldp<NP>(z, A.xi + 2 * Vp + v);
        else
#pragma unroll
            for (int p = 0; p < NP; ++p) z[p] = f2(0.0f);
        ldp<NP>(w, A.w + v);
        ldp<NP>(mr, A.mref + v);
    }
    // from a shared-memory copy [x | y | (z) | w | mref], Vp each (dv_table32)
    __device__ __forceinline__ void load_tab(const float* tab, int Vp, int v0, int lane) {
        const int v = v0 + lane * NPL;
        ldp<NP>(x, tab + v);
        ldp<NP>(y, tab + Vp + v);
        if (D == 3) ldp<NP>(z, tab + 2 * Vp + v);
        else
#pragma unroll
            for (int p = 0; p < NP; ++p) z[p] = f2(0.0f);
        ldp<NP>(w, tab + D * Vp + v);
        ldp<NP>(mr, tab + (D + 1) * Vp + v);
    }
};

// The velocity constants of Lane32 for all Vp velocities, copied by a block
// into shared memory (caller synchronises); its size in bytes.
__host__ __device__ inline size_t dv_table32_bytes(int D, int Vp) { return (size_t)(D + 2) * Vp * sizeof(float); }
template <int D>
__device__ __forceinline__ void dv_table32(const FusedArgs<float>& A, float* tab) {
    const int Vp = A.b.Vp;
    for (int q = threadIdx.x; q < (D + 2) * Vp; q += blockDim.x) {
        const int k = q / Vp, v = q - k * Vp;
        tab[q] = k < D ? A.xi[k * Vp + v] : (k == D ? A.w[v] : A.mref[v]);
    }
}

// Shakhov relaxation in deviation form: out = G - a (G + Mref) + a g^S, with
//   a g^S = aA e [1 + phi u],   e = exp(-c^2 / 2RT),  u = c^2/RT - (D+2),
//   a h^S = RT [aA e phi ((K+3-D) u + 6 - 2D) + aA e (K+3-D)]
// (phi = the Shakhov heat-flux term q'.c; the h form is the reference's
// ((c^2/RT - D)(K+3-D) - 2K) regrouped about u, so that g and h share u).
template <int D, bool H>
struct Eq32 {
    float ux, uy, uz, kexp, invRT, qx, qy, qz, a, aA, KDRT, C0RT, hf;
    __device__ __forceinline__ void load(const float4* q, int K, float hrefFac) {  // an eq_table entry
        const float4 b0 = q[0], b1 = q[1], b2 = q[2];
        ux = b0.x; uy = b0.y; uz = b0.z; kexp = b0.w;
        invRT = b1.x; qx = b1.y; qy = b1.z; qz = b1.w;
        a = b2.x;
        aA = b2.y;
        const float RT = b2.z;
        KDRT = (float)(K + 3 - D) * RT;
        C0RT = (float)(6 - 2 * D) * RT;
        hf = hrefFac;
    }
    template <int NPL>
    __device__ __forceinline__ void relax(const Lane32<D, NPL>& L, int p, float2& g, float2& h) const {
        const float2 cx = sub2(L.x[p], f2(ux)), cy = sub2(L.y[p], f2(uy));
        float2 c2 = fma2(cy, cy, mul2(cx, cx));
        float2 phi = fma2(cy, f2(qy), mul2(cx, f2(qx)));
        if (D == 3) {
            const float2 cz = sub2(L.z[p], f2(uz));
            c2 = fma2(cz, cz, c2);
            phi = fma2(cz, f2(qz), phi);
        }
        const float2 t = mul2(c2, f2(kexp));
        const float2 e = mul2(make_float2(ex2f(t.x), ex2f(t.y)), f2(aA));
        const float2 u = fma2(c2, f2(invRT), f2(-(float)(D + 2)));
        const float2 ep = mul2(e, phi);
        const float2 ags = fma2(ep, u, e);
        g = fma2(f2(-a), add2(g, L.mr[p]), add2(g, ags));
        if (H) {
            const float2 ahs = fma2(ep, fma2(u, f2(KDRT), f2(C0RT)), mul2(e, f2(KDRT)));
            h = fma2(f2(-a), add2(h, mul2(L.mr[p], f2(hf))), add2(h, ahs));
        }
    }
};


// Asynchronous global -> shared copies (each lane copies, and later reads,
// only its own NPL floats of a row, so a lane's wait_group is all the
// ordering it needs).
__device__ __forceinline__ void cp_async_row(float* dst, const float* src, int npl) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(dst);
    if (npl == 4) asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(src) : "memory");
    else asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

// Raw g~ (and h~) rows of T u H1 for the DV chunk at v0 into shared memory,
// 16-byte asynchronous copies (one commit group).  Warp w copies rows w,
// w + NW, ... -- the rows it relaxes -- so that after its own wait_group and
// a __syncwarp it may relax them without a block barrier.
// Rows of one DV chunk in shared memory: row r of field f (0 g, 1 h) at
// t[f] + r KC for the cells of T (r < nT) and at hh[f] + (r - nT) KC for the
// halo; hh[f] = t[f] + nT KC when the halo follows T in one block.
struct Rows32 {
    float* t[2];
    float* hh[2];
    int nT;
    template <bool SPLIT>  // halo rows apart from the rows of T
    __device__ __forceinline__ float* row(int f, int r, int KC) const {
        if (!SPLIT) return t[f] + r * KC;
        return r < nT ? t[f] + r * KC : hh[f] + (r - nT) * KC;
    }
};

template <int NPL, bool H, int NW, bool SPLIT>
__device__ __forceinline__ void issue_rows32(const FusedArgs<float>& A, const TileHdr& hd, const int* C,
                                             const Rows32& rs, int v0, int warp, int lane, int r0, int r1) {
    constexpr int KC = 32 * NPL, SEG = KC / 4;
    for (int r = warp; r < hd.nT2; r += NW) {
        if (r < r0 || r >= r1) continue;
        const size_t gr = (size_t)C[r] * A.b.Vp + v0;
        float* dg = rs.row<SPLIT>(0, r, KC);
        float* dh = H ? rs.row<SPLIT>(1, r, KC) : nullptr;
        for (int sgm = lane; sgm < SEG; sgm += 32) {
            cp_async_row(dg + sgm * 4, A.gT + gr + sgm * 4, 4);
            if (H) cp_async_row(dh + sgm * 4, A.hT + gr + sgm * 4, 4);
        }
    }
    cp_async_commit();
}

// gbar+ = relaxation of the raw rows in place (shared memory only).
template <int D, bool H, int NPL, int NW, bool SPLIT>
__device__ __forceinline__ void relax_rows32(const FusedArgs<float>& A, const TileHdr& hd, const float4* ceq,
                                             const Lane32<D, NPL>& L, int lane, int warp, const Rows32& rs) {
    constexpr int KC = 32 * NPL, NP = NPL / 2;
    for (int r = warp; r < hd.nT2; r += NW) {
        float2 g[NP], h[NP];
        float* sg = rs.row<SPLIT>(0, r, KC);
        float* sh = H ? rs.row<SPLIT>(1, r, KC) : sg;
        ldp<NP>(g, sg + lane * NPL);
        if (H) ldp<NP>(h, sh + lane * NPL);
        Eq32<D, H> e;
        e.load(ceq + 3 * r, A.b.K, A.hrefFac);
#pragma unroll
        for (int p = 0; p < NP; ++p) {
            if (!H) h[p] = f2(0.f);
            e.relax(L, p, g[p], h[p]);
        }
        stp<NP>(sg + lane * NPL, g);
        if (H) stp<NP>(sh + lane * NPL, h);
    }
}

// Face record + geometry in registers.
struct Face32 {
    TileFace r;
    float Sx, Sy, Sz, iVo, dOx, dOy, dOz, iVn, dNx, dNy, dNz;
    int plain;  // stencil entries of the owner (bits 0-7) and neighbour (8-15) side when all are cell rows, else 0
    __device__ __forceinline__ void load(const int4* p) {  // a staged face record
        const int4 a = p[0], b = p[1];
        r.ownL = a.x; r.neiL = a.y; r.a = a.z; r.w = a.w;
        r.stO0 = b.x; r.stO1 = b.y; r.stN0 = b.z; r.stN1 = b.w;
        const float4* g = reinterpret_cast<const float4*>(p + 2);
        const float4 g0 = g[0], g1 = g[1], g2 = g[2];
        Sx = g0.x; Sy = g0.y; Sz = g0.z; iVo = g0.w;
        dOx = g1.x; dOy = g1.y; dOz = g1.z; iVn = g1.w;
        dNx = g2.x; dNy = g2.y; dNz = g2.z;
        plain = __float_as_int(g2.w);
    }
    template <int D, int NPL>
    __device__ __forceinline__ float2 xs(const Lane32<D, NPL>& L, int p) const {
        float2 s = fma2(L.y[p], f2(Sy), mul2(L.x[p], f2(Sx)));
        if (D == 3) s = fma2(L.z[p], f2(Sz), s);
        return s;
    }
};

// One side's reconstruction sum over its stencil entry k:
//   acc += beta (phi_o - phi_u),  beta = L.(d_u - xi dt/2),
// with the neighbour row (or the lagged wall gradient) read for all pairs.
// PLAIN: the entry is known to be a cell row (no wall branch).
template <int D, bool H, int NP, bool GRAD, bool PLAIN = false>
__device__ __forceinline__ void side_entry(const FusedArgs<float>& A, const float4* E, int e, float dx, float dy, float dz,
                                           const float2 (&cu)[NP], const float2 (&hu)[NP], const float* sg,
                                           const float* sh, int col, int v0, const float2* xx, const float2* xy,
                                           const float2* xz, float2 (&acc)[NP], float2 (&acch)[NP],
                                           float2 (&gw)[D][NP], float2 (&hw)[D][NP]) {
    constexpr int KC = 64 * NP;
    const float4 ent = E[e];
    const int o = __float_as_int(ent.w);
    const float hdt = -0.5f * A.dt;
    float al = fmaf(ent.y, dy, ent.x * dx);
    if (D == 3) al = fmaf(ent.z, dz, al);
    const float2 lx = f2(hdt * ent.x), ly = f2(hdt * ent.y), lz = f2(hdt * ent.z);
    float2 r[NP], q[NP];
    if (PLAIN || o >= 0) {
        ldp<NP>(r, sg + o * KC + col);
        if (H) ldp<NP>(q, sh + o * KC + col);
    } else {  // wall entry: phi_b - phi_P = G_b / deltaCoeff
        const int wf = -o - 1;
        const float idc = A.wall4[wf].y;
        float2 tg[NP], th[NP];
        ldp<NP>(tg, A.Gbg + (size_t)wf * A.b.Vp + v0 + col);
        if (H) ldp<NP>(th, A.Gbh + (size_t)wf * A.b.Vp + v0 + col);
#pragma unroll
        for (int p = 0; p < NP; ++p) {
            r[p] = fma2(tg[p], f2(idc), cu[p]);
            if (H) q[p] = fma2(th[p], f2(idc), hu[p]);
        }
    }
#pragma unroll
    for (int p = 0; p < NP; ++p) {
        float2 beta = fma2(ly, xy[p], fma2(lx, xx[p], f2(al)));
        if (D == 3) beta = fma2(lz, xz[p], beta);
        const float2 dg = sub2(r[p], cu[p]);
        acc[p] = fma2(beta, dg, acc[p]);
        float2 dh = f2(0.0f);
        if (H) {
            dh = sub2(q[p], hu[p]);
            acch[p] = fma2(beta, dh, acch[p]);
        }
        if (GRAD) {
            gw[0][p] = fma2(f2(ent.x), dg, gw[0][p]);
            gw[1][p] = fma2(f2(ent.y), dg, gw[1][p]);
            if (D == 3) gw[2][p] = fma2(f2(ent.z), dg, gw[2][p]);
            if (H) {
                hw[0][p] = fma2(f2(ent.x), dh, hw[0][p]);
                hw[1][p] = fma2(f2(ent.y), dh, hw[1][p]);
                if (D == 3) hw[2][p] = fma2(f2(ent.z), dh, hw[2][p]);
            }
        }
    }
}

// Upwind weight of the owner side of a face for one velocity from s = xi.S:
// 1 for s > 0, 0 for s < 0, 1/2 for s == 0 (one saturating FMA; |s| below
// 2^-101 would count as a partial tie, far below any xi.S of a real face).
__device__ __forceinline__ float2 upwind_w2(float2 s) {
    return make_float2(__saturatef(fmaf(s.x, 0x1p100f, 0.5f)), __saturatef(fmaf(s.y, 0x1p100f, 0.5f)));
}
// w go + (1 - w) gn, exactly go for w = 1 and gn for w = 0.
__device__ __forceinline__ float2 blend2(float2 w, float2 go, float2 gn) {
    return fma2(w, go, mul2(sub2(f2(1.0f), w), gn));
}

// Upwind reconstruction gbar_f = gbar+_u + sum_e (L_e.(d_u - xi dt/2)) (gbar+_o(e) - gbar+_u)
// for the lane's velocities.  Both sides are summed (packed, no per-entry
// selects) and each velocity takes the owner side when xi.S > 0, the
// neighbour side when xi.S < 0 and their average when xi.S == 0.  Walls have
// only the owner side; there the owner gradient itself is also returned.
template <int D, bool H, int NPL, bool WALL>
__device__ __forceinline__ void recon32(const FusedArgs<float>& A, const float4* E, const Face32& F, const Lane32<D, NPL>& L,
                                        const float* sg, const float* sh, int lane, int v0, const float2* xs,
                                        float2 (&gf)[NPL / 2], float2 (&hf)[NPL / 2], float2 (&gw)[D][NPL / 2],
                                        float2 (&hw)[D][NPL / 2]) {
    constexpr int KC = 32 * NPL, NP = NPL / 2;
    const int col = lane * NPL;
    float2 cO[NP], hO[NP], cN[NP], hN[NP];
    float2 aO[NP], ahO[NP], aN[NP], ahN[NP];
    ldp<NP>(cO, sg + F.r.ownL * KC + col);
    if (H) ldp<NP>(hO, sh + F.r.ownL * KC + col);
#pragma unroll
    for (int p = 0; p < NP; ++p) {
        aO[p] = f2(0.f); ahO[p] = f2(0.f); aN[p] = f2(0.f); ahN[p] = f2(0.f);
        if (!H) { hO[p] = f2(0.f); hN[p] = f2(0.f); }
#pragma unroll
        for (int k = 0; k < D; ++k) { gw[k][p] = f2(0.f); hw[k][p] = f2(0.f); }
    }
    if (WALL) {
        for (int e = F.r.stO0; e < F.r.stO1; ++e)
            side_entry<D, H, NP, true>(A, E, e, F.dOx, F.dOy, F.dOz, cO, hO, sg, sh, col, v0, L.x, L.y, L.z, aO, ahO, gw, hw);
#pragma unroll
        for (int p = 0; p < NP; ++p) {
            gf[p] = add2(cO[p], aO[p]);
            if (H) hf[p] = add2(hO[p], ahO[p]);
        }
        return;
    }
    ldp<NP>(cN, sg + F.r.neiL * KC + col);
    if (H) ldp<NP>(hN, sh + F.r.neiL * KC + col);
    float2 dw[D][NP], dhw[D][NP];
    // owner and neighbour entries interleaved: two independent accumulation chains
    const int nO = F.r.stO1 - F.r.stO0, nN = F.r.stN1 - F.r.stN0;
    for (int k = 0; k < max(nO, nN); ++k) {
        if (k < nO)
            side_entry<D, H, NP, false>(A, E, F.r.stO0 + k, F.dOx, F.dOy, F.dOz, cO, hO, sg, sh, col, v0, L.x, L.y, L.z, aO,
                                        ahO, gw, hw);
        if (k < nN)
            side_entry<D, H, NP, false>(A, E, F.r.stN0 + k, F.dNx, F.dNy, F.dNz, cN, hN, sg, sh, col, v0, L.x, L.y, L.z, aN,
                                        ahN, dw, dhw);
    }
#pragma unroll
    for (int p = 0; p < NP; ++p) {
        const float2 w = upwind_w2(xs[p]);
        gf[p] = blend2(w, add2(cO[p], aO[p]), add2(cN[p], aN[p]));
        if (H) hf[p] = blend2(w, add2(hO[p], ahO[p]), add2(hN[p], ahN[p]));
    }
}

// recon32 for an internal face whose two stencils are plain (NE cell-row
// entries each, no wall entry): both sides summed with the entry loop
// unrolled, then the per-velocity upwind blend.
template <int D, bool H, int NPL, int NE>
__device__ __forceinline__ void recon_plain32(const FusedArgs<float>& A, const float4* E, const Face32& F,
                                              const Lane32<D, NPL>& L, const float* sg, const float* sh, int lane,
                                              int v0, const float2* xs, float2 (&gf)[NPL / 2], float2 (&hf)[NPL / 2]) {
    constexpr int KC = 32 * NPL, NP = NPL / 2;
    const int col = lane * NPL;
    float2 cO[NP], hO[NP], cN[NP], hN[NP], aO[NP], ahO[NP], aN[NP], ahN[NP], gw[D][NP], hw[D][NP];
    ldp<NP>(cO, sg + F.r.ownL * KC + col);
    ldp<NP>(cN, sg + F.r.neiL * KC + col);
    if (H) {
        ldp<NP>(hO, sh + F.r.ownL * KC + col);
        ldp<NP>(hN, sh + F.r.neiL * KC + col);
    }
#pragma unroll
    for (int p = 0; p < NP; ++p) {
        aO[p] = f2(0.f); ahO[p] = f2(0.f); aN[p] = f2(0.f); ahN[p] = f2(0.f);
        if (!H) { hO[p] = f2(0.f); hN[p] = f2(0.f); }
    }
#pragma unroll
    for (int k = 0; k < NE; ++k) {
        side_entry<D, H, NP, false, true>(A, E, F.r.stO0 + k, F.dOx, F.dOy, F.dOz, cO, hO, sg, sh, col, v0, L.x, L.y,
                                          L.z, aO, ahO, gw, hw);
        side_entry<D, H, NP, false, true>(A, E, F.r.stN0 + k, F.dNx, F.dNy, F.dNz, cN, hN, sg, sh, col, v0, L.x, L.y,
                                          L.z, aN, ahN, gw, hw);
    }
#pragma unroll
    for (int p = 0; p < NP; ++p) {
        const float2 w = upwind_w2(xs[p]);
        gf[p] = blend2(w, add2(cO[p], aO[p]), add2(cN[p], aN[p]));
        hf[p] = H ? blend2(w, add2(hO[p], ahO[p]), add2(hN[p], ahN[p])) : f2(0.f);
    }
}

// recon_one32 for a plain side of NE cell-row entries (loop unrolled).
template <int D, bool H, int NPL, int NE>
__device__ __forceinline__ void recon_one_plain32(const FusedArgs<float>& A, const float4* E, int e0, int lu, float dx,
                                                  float dy, float dz, const Lane32<D, NPL>& L, const float* sg,
                                                  const float* sh, int lane, int v0, float2 (&gv)[NPL / 2],
                                                  float2 (&hv)[NPL / 2]) {
    constexpr int KC = 32 * NPL, NP = NPL / 2;
    const int col = lane * NPL;
    float2 c[NP], hc[NP], ac[NP], ah[NP], gw[D][NP], hw[D][NP];
    ldp<NP>(c, sg + lu * KC + col);
    if (H) ldp<NP>(hc, sh + lu * KC + col);
#pragma unroll
    for (int p = 0; p < NP; ++p) {
        ac[p] = f2(0.f);
        ah[p] = f2(0.f);
        if (!H) hc[p] = f2(0.f);
    }
#pragma unroll
    for (int k = 0; k < NE; ++k)
        side_entry<D, H, NP, false, true>(A, E, e0 + k, dx, dy, dz, c, hc, sg, sh, col, v0, L.x, L.y, L.z, ac, ah, gw,
                                          hw);
#pragma unroll
    for (int p = 0; p < NP; ++p) {
        gv[p] = add2(c[p], ac[p]);
        hv[p] = H ? add2(hc[p], ah[p]) : f2(0.f);
    }
}

// Deviation moments of the lane's velocities about ur into its slots
// (mask: per-velocity inclusion, used on walls for the outgoing half);
// ASSIGN: the slots of the moments are set, else added to.
template <int D, bool H, int NPL, int NS, bool ASSIGN = false>
__device__ __forceinline__ void mom32(float (&m)[NS], const Lane32<D, NPL>& L, const float* ur,
                                      const float2 (&g)[NPL / 2], const float2 (&h)[NPL / 2], const float2* mask) {
    using SL = Slots<D, H>;
    constexpr int NP = NPL / 2;
    float2 m2[NS];
#pragma unroll
    for (int p = 0; p < NP; ++p) {  // pair 0 sets the packed sums, the others add
        const bool first = p == 0;
        const float2 c[3] = {sub2(L.x[p], f2(ur[0])), sub2(L.y[p], f2(ur[1])),
                             D == 3 ? sub2(L.z[p], f2(ur[2])) : f2(0.f)};
        float2 wg = mul2(L.w[p], g[p]);
        if (mask) wg = mul2(wg, mask[p]);
        m2[0] = first ? wg : add2(m2[0], wg);
        float2 c2 = mul2(c[0], c[0]);
#pragma unroll
        for (int i = 1; i < D; ++i) c2 = fma2(c[i], c[i], c2);
#pragma unroll
        for (int i = 0; i < D; ++i) {
            const float2 t = mul2(wg, c[i]);
            m2[SL::M1 + i] = first ? t : add2(m2[SL::M1 + i], t);
#pragma unroll
            for (int k = i; k < D; ++k) {
                const int j = SL::M2 + sym<D>(i, k);
                m2[j] = first ? mul2(t, c[k]) : fma2(t, c[k], m2[j]);
            }
            m2[SL::M3 + i] = first ? mul2(t, c2) : fma2(t, c2, m2[SL::M3 + i]);
        }
        if (H) {
            float2 wh = mul2(L.w[p], h[p]);
            if (mask) wh = mul2(wh, mask[p]);
            m2[SL::H0] = first ? wh : add2(m2[SL::H0], wh);
#pragma unroll
            for (int i = 0; i < D; ++i) m2[SL::H1 + i] = first ? mul2(wh, c[i]) : fma2(wh, c[i], m2[SL::H1 + i]);
        }
    }
#pragma unroll
    for (int s = 0; s < SL::NM; ++s) {
        if (ASSIGN) m[s] = m2[s].x + m2[s].y;
        else m[s] += m2[s].x + m2[s].y;
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

// Face macros (FP64) from the deviation moment totals M of face a (wall w or
// -1) about its reference velocity u4: P4 Maxwell-wall density, P5 incoming
// wall moments, P6 face macros, wall heat flux and stress; then the face
// equilibrium table and the next reference velocity.
template <int D, bool H>
__device__ __forceinline__ void finalize_face32(const FusedArgs<float>& A, int a, int w, float4 u4, double* M) {
    using SL = Slots<D, H>;
    constexpr int NS = SL::NS;
    const StepArgs& b = A.b;
    const double ur[3] = {u4.x, u4.y, u4.z};
    double rw = 0.0;
    if (w >= 0) {  // outgoing: deviation + reference parts; incoming: rho_w * Mw
        const double* RO = A.wallRefOut + (size_t)w * NS;
        for (int s = 0; s <= SL::FLUX; ++s) M[s] += RO[s];
        rw = M[SL::FLUX] / b.incAbs[w];
        for (int s = 0; s < SL::NM; ++s) M[s] += rw * A.Min[(size_t)w * NS + s];
    } else {
        double Rm[NS];
        ref_moments_about<D, H>(A.refMom, ur, Rm);
        for (int s = 0; s < SL::NM; ++s) M[s] += Rm[s];
    }
    for (int s = 0; s < SL::NM; ++s) M[s] *= A.invGscale;
    double rho, U[3], T, tau, qr[3];
    macros_from_moments<D, H, true>(M, ur, b, rho, U, T, tau, qr);
    const double fac = 2.0 * tau / (2.0 * tau + 0.5 * b.dt * b.Pr);
    double q[3] = {fac * qr[0], fac * qr[1], fac * qr[2]};
    b.rhoF[a] = rho;
    b.TF[a] = T;
    b.tauF[a] = tau;
    for (int k = 0; k < 3; ++k) { b.UF[3 * a + k] = U[k]; b.qF[3 * a + k] = q[k]; }
    float* blk = A.fc + (size_t)a * kNCoef;
    write_coef<D>(blk, rho, U, T, q, tau, b, A.gscale);
    if (A.feqT) eq_table(A.feqT + 3 * (size_t)a, blk, face_weight(A.dt, blk));
    if (w < 0) {
        A.uref4[a] = make_float4((float)U[0], (float)U[1], (float)U[2], 0.0f);
        return;
    }
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
            double sv = 0.0;
            if (i < D && j < D) {
                const double m2 = M[SL::M2 + (i <= j ? sym<D>(i, j) : sym<D>(j, i))];
                sv = m2 + ur[i] * M[SL::M1 + j] + ur[j] * M[SL::M1 + i] + ur[i] * ur[j] * M[0];
            }
            b.stressWall[9 * w + 3 * i + j] = fs * sv;
        }
}

// ---------------------------------------------------------------- sweep A, face sides
// One-sided upwind reconstruction from cell u (local row lu, stencil entries
// [e0,e1) of u, d = Cf - C_u): val = gbar+_u + sum_e L_e.(d - xi dt/2) (gbar+_e - gbar+_u).
template <int D, bool H, int NPL>
__device__ __forceinline__ void recon_one32(const FusedArgs<float>& A, const float4* E, int e0, int e1, int lu,
                                            float dx, float dy, float dz, const Lane32<D, NPL>& L, const float* sg,
                                            const float* sh, int lane, int v0, float2 (&gv)[NPL / 2],
                                            float2 (&hv)[NPL / 2]) {
    constexpr int KC = 32 * NPL, NP = NPL / 2;
    const int col = lane * NPL;
    float2 c[NP], hc[NP], ac[NP], ah[NP], gw[D][NP], hw[D][NP];
    ldp<NP>(c, sg + lu * KC + col);
    if (H) ldp<NP>(hc, sh + lu * KC + col);
#pragma unroll
    for (int p = 0; p < NP; ++p) {
        ac[p] = f2(0.f);
        ah[p] = f2(0.f);
        if (!H) hc[p] = f2(0.f);
    }
    for (int e = e0; e < e1; ++e)
        side_entry<D, H, NP, false>(A, E, e, dx, dy, dz, c, hc, sg, sh, col, v0, L.x, L.y, L.z, ac, ah, gw, hw);
#pragma unroll
    for (int p = 0; p < NP; ++p) {
        gv[p] = add2(c[p], ac[p]);
        hv[p] = H ? add2(hc[p], ah[p]) : f2(0.f);
    }
}

// Sweep A on tiles with a one-ring halo (rows of T u H1).  Every face touching
// T is visited.  A face with both cells in T, and every wall face of T, is
// complete here; for a face across the tile boundary only the side whose cell
// is in T is reconstructed (its gradient needs T u H1 only): the velocities
// for which that cell is upwind, plus half of the ties (xi.S == 0) in the
// moments.  The tile on the other side adds the rest, so every face side is
// reconstructed exactly once.  Per-side moment totals go to faceMom[a][side]
// (side 0: owner or complete, side 1: neighbour) and k_face_macros32 forms the
// face macros.  Face values are stored for the velocities this side owns
// (tie values are never read: their flux is zero).  Raw rows of the next DV
// chunk stream into the second row buffer while this chunk's faces run.
// Least-squares gradients of the cells of T for the chunk (one warp per cell):
// grad_c = sum_e L_e (gbar+_e - gbar+_c), a wall entry contributing
// L_b G_b / deltaCoeff (the lagged boundary gradient).
template <int D, bool H, int NPL, int NW>
__device__ __forceinline__ void cell_gradients32(const FusedArgs<float>& A, const TileHdr& hd, const TileMeta32& tm,
                                                 const Rows32& rs, float* gbuf, int lane, int warp, int v0) {
    constexpr int KC = 32 * NPL, NP = NPL / 2, NR = H ? 2 : 1;
    const int col = lane * NPL, Vp = A.b.Vp;
    for (int lc = warp; lc < hd.nT; lc += NW) {
        float2 c[NP], hc[NP], gg[D][NP], hg[D][NP];
        ldp<NP>(c, rs.row<true>(0, lc, KC) + col);
        if (H) ldp<NP>(hc, rs.row<true>(1, lc, KC) + col);
#pragma unroll
        for (int k = 0; k < D; ++k)
#pragma unroll
            for (int p = 0; p < NP; ++p) { gg[k][p] = f2(0.f); hg[k][p] = f2(0.f); }
        for (int e = tm.S[lc]; e < tm.S[lc + 1]; ++e) {
            const float4 ent = tm.E[e];
            const int o = __float_as_int(ent.w);
            const float Lk[3] = {ent.x, ent.y, ent.z};
            float2 dg[NP], dh[NP];
            if (o >= 0) {
                float2 r[NP], q[NP];
                ldp<NP>(r, rs.row<true>(0, o, KC) + col);
                if (H) ldp<NP>(q, rs.row<true>(1, o, KC) + col);
#pragma unroll
                for (int p = 0; p < NP; ++p) {
                    dg[p] = sub2(r[p], c[p]);
                    if (H) dh[p] = sub2(q[p], hc[p]);
                }
            } else {
                const int wf = -o - 1;
                const float idc = A.wall4[wf].y;
                float2 tg[NP], th[NP];
                ldp<NP>(tg, A.Gbg + (size_t)wf * Vp + v0 + col);
                if (H) ldp<NP>(th, A.Gbh + (size_t)wf * Vp + v0 + col);
#pragma unroll
                for (int p = 0; p < NP; ++p) {
                    dg[p] = mul2(tg[p], f2(idc));
                    if (H) dh[p] = mul2(th[p], f2(idc));
                }
            }
#pragma unroll
            for (int k = 0; k < D; ++k)
#pragma unroll
                for (int p = 0; p < NP; ++p) {
                    gg[k][p] = fma2(f2(Lk[k]), dg[p], gg[k][p]);
                    if (H) hg[k][p] = fma2(f2(Lk[k]), dh[p], hg[k][p]);
                }
        }
#pragma unroll
        for (int k = 0; k < D; ++k) {
            stp<NP>(gbuf + ((lc * D + k) * NR) * KC + col, gg[k]);
            if (H) stp<NP>(gbuf + ((lc * D + k) * NR + 1) * KC + col, hg[k]);
        }
    }
}

// Face value from cell lc of T: gbar+_c + grad_c . (d - xi dt/2); optionally
// the normal gradient grad_c . nh (wall update).
template <int D, bool H, int NPL>
__device__ __forceinline__ void side_value_g(const Lane32<D, NPL>& L, const float* sg, const float* sh,
                                             const float* gbuf, int lc, const float* d, float dt, int col,
                                             float2 (&gv)[NPL / 2], float2 (&hv)[NPL / 2]) {
    constexpr int KC = 32 * NPL, NP = NPL / 2, NR = H ? 2 : 1;
    ldp<NP>(gv, sg + lc * KC + col);
    if (H) ldp<NP>(hv, sh + lc * KC + col);
    else
#pragma unroll
        for (int p = 0; p < NP; ++p) hv[p] = f2(0.f);
    const float2 hdt = f2(-0.5f * dt);
#pragma unroll
    for (int k = 0; k < D; ++k) {
        float2 gk[NP], hk[NP];
        ldp<NP>(gk, gbuf + ((lc * D + k) * NR) * KC + col);
        if (H) ldp<NP>(hk, gbuf + ((lc * D + k) * NR + 1) * KC + col);
        const float2* xk = k == 0 ? L.x : (k == 1 ? L.y : L.z);
#pragma unroll
        for (int p = 0; p < NP; ++p) {
            const float2 beta = fma2(xk[p], hdt, f2(d[k]));
            gv[p] = fma2(gk[p], beta, gv[p]);
            if (H) hv[p] = fma2(hk[p], beta, hv[p]);
        }
    }
}

template <int D, bool H, int NPL, int NW, bool GR>
__device__ __forceinline__ void face_sides_body(const FusedArgs<float>& A, int tile, unsigned char* smem) {
    using SL = Slots<D, H>;
    constexpr int NS = SL::NS, KC = 32 * NPL, NP = NPL / 2;
    const TileHdr hd = A.hdr[tile];
    const StepArgs& b = A.b;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int Vp = b.Vp, col = lane * NPL;
    using LY = SmemLayout32<D, H, NPL, GR>;
    // the row buffer of chunk parity bf
    float* const rowBase = reinterpret_cast<float*>(smem);
    const size_t nTK = (size_t)hd.nT * KC, nHK = (size_t)(hd.nT2 - hd.nT) * KC;
    auto rowsOf = [&](int bf) {
        Rows32 r;
        r.nT = hd.nT;
        if (GR) {  // [T g,h (buffer 0)][T g,h (buffer 1)][halo g,h]
            r.t[0] = rowBase + bf * (H ? 2 : 1) * nTK;
            r.t[1] = r.t[0] + nTK;
            r.hh[0] = rowBase + 2 * (H ? 2 : 1) * nTK;
            r.hh[1] = r.hh[0] + nHK;
        } else {  // per buffer: g rows of T u H1, then h rows
            r.t[0] = rowBase + bf * (H ? 2 : 1) * (nTK + nHK);
            r.t[1] = r.t[0] + nTK + nHK;
            r.hh[0] = r.t[0] + nTK;
            r.hh[1] = r.t[1] + nTK;
        }
        return r;
    };
    float* gbuf = reinterpret_cast<float*>(smem + LY::rowBlock(hd.nT2, hd.nT));  // GR: gradients of T
    Acc<float>* mom = reinterpret_cast<Acc<float>*>(smem + LY::mom(hd.nT2, hd.nT));
    for (int i = threadIdx.x; i < hd.nFB * NS; i += NW * 32) mom[i].zero();
    const TileMeta32 tm = stage_meta<NW * 32>(A, hd, tile, smem + LY::meta(hd.nT2, hd.nFB, hd.nT));
    float4* sU = tm.dyn;            // [nFB] face Uref
    float4* ceq = tm.dyn + hd.nFB;  // [nT2][3] cell equilibria
    __syncthreads();
#if defined(DUGKS_CHECKED) && DUGKS_CHECKED
    check_tile_meta32<NW * 32>(A, hd, smem + LY::meta(hd.nT2, hd.nFB, hd.nT));
    __syncthreads();
#endif
    for (int i = threadIdx.x; i < hd.nFB; i += NW * 32) sU[i] = A.uref4[tm.F[5 * i].z];
    for (int i = threadIdx.x; i < hd.nT2; i += NW * 32) {
        const float* blk = A.cc + (size_t)tm.C[i] * kNCoef;
        eq_table(ceq + 3 * i, blk, cell_weight(A.dt, blk));
    }
    issue_rows32<NPL, H, NW, GR>(A, hd, tm.C, rowsOf(0), 0, warp, lane, 0, hd.nT2);
    const int nChunks = Vp / KC;
    const int myslot = slot_of<NS>(lane);
    const bool writer = NS == 16 ? (lane & 1) == 0 : true;
    __syncthreads();  // face Uref and cell equilibria

    // One block barrier per chunk: a warp relaxes the rows it copied itself
    // as soon as its copies have landed (a warp still in the previous
    // chunk's faces reads the other buffer), the barrier after the
    // relaxation releases the faces, and only then are the next chunk's
    // rows copied into the buffer that the previous chunk's faces read.
    for (int ch = 0; ch < nChunks; ++ch) {
        const int v0 = ch * KC;
        Lane32<D, NPL> L;
        L.load(A, v0, lane);
        cp_async_wait<0>();
        __syncwarp();
        const Rows32 rc = rowsOf(ch & 1);
        float* cg = rc.t[0];
        float* chh = rc.t[1];
        relax_rows32<D, H, NPL, NW, GR>(A, hd, ceq, L, lane, warp, rc);
        __syncthreads();
        // next chunk's rows: those of T now (the faces of this chunk read the
        // other buffer); with per-cell gradients the halo rows, single
        // buffered, only after the gradient pass has read them
        if (ch + 1 < nChunks)
            issue_rows32<NPL, H, NW, GR>(A, hd, tm.C, rowsOf((ch + 1) & 1), v0 + KC, warp, lane, 0, GR ? hd.nT : hd.nT2);
        if (GR) {
            cell_gradients32<D, H, NPL, NW>(A, hd, tm, rc, gbuf, lane, warp, v0);
            __syncthreads();
            if (ch + 1 < nChunks)
                issue_rows32<NPL, H, NW, GR>(A, hd, tm.C, rowsOf((ch + 1) & 1), v0 + KC, warp, lane, hd.nT, hd.nT2);
        }
        for (int lf = warp; lf < hd.nFB; lf += NW) {
            Face32 F;
            F.load(tm.F + 5 * lf);
            const float4 u4 = sU[lf];
            const float ur[3] = {u4.x, u4.y, u4.z};
            float2 xs[NP];
#pragma unroll
            for (int p = 0; p < NP; ++p) xs[p] = F.xs<D, NPL>(L, p);
            float2 gf[NP], hf[NP], gw[D][NP], hw[D][NP];
            float m[NS];
#pragma unroll
            for (int s = 0; s < NS; ++s) m[s] = 0.0f;
            const size_t fi = (size_t)F.r.a * Vp + v0 + col;
            const float dO[3] = {F.dOx, F.dOy, F.dOz}, dN[3] = {F.dNx, F.dNy, F.dNz};
            if (F.r.w >= 0) {
                if (GR) {  // boundary: owner side; gw = the owner's gradient (for grad . n)
                    side_value_g<D, H, NPL>(L, cg, chh, gbuf, F.r.ownL, dO, A.dt, col, gf, hf);
#pragma unroll
                    for (int k = 0; k < D; ++k) {
                        ldp<NP>(gw[k], gbuf + ((F.r.ownL * D + k) * (H ? 2 : 1)) * KC + col);
                        if (H) ldp<NP>(hw[k], gbuf + ((F.r.ownL * D + k) * 2 + 1) * KC + col);
                    }
                } else {
                    recon32<D, H, NPL, true>(A, tm.E, F, L, cg, chh, lane, v0, xs, gf, hf, gw, hw);
                }
                float2 gn[NP], hn[NP], use[NP];
                float fl = 0.0f;
#pragma unroll
                for (int p = 0; p < NP; ++p) {
                    gn[p] = fma2(gw[1][p], f2(F.dNy), mul2(gw[0][p], f2(F.dNx)));
                    if (D == 3) gn[p] = fma2(gw[2][p], f2(F.dNz), gn[p]);
                    if (H) {
                        hn[p] = fma2(hw[1][p], f2(F.dNy), mul2(hw[0][p], f2(F.dNx)));
                        if (D == 3) hn[p] = fma2(hw[2][p], f2(F.dNz), hn[p]);
                    }
                    use[p] = make_float2(xs[p].x > 0.f ? 1.f : 0.f, xs[p].y > 0.f ? 1.f : 0.f);
                    const float2 fx = mul2(mul2(mul2(L.w[p], xs[p]), gf[p]), use[p]);
                    fl += fx.x + fx.y;
                }
                m[SL::FLUX] = fl;
                const size_t wi = (size_t)F.r.w * Vp + v0 + col;
                stp<NP>(A.Gbgn + wi, gn);
                if (H) stp<NP>(A.Gbhn + wi, hn);
                mom32<D, H, NPL, NS, true>(m, L, ur, gf, hf, use);
                stp<NP>(A.gF + fi, gf);
                if (H) stp<NP>(A.hF + fi, hf);
            } else if (F.r.ownL < hd.nT && F.r.neiL < hd.nT) {  // both sides in T: complete
                if (GR) {
                    float2 go[NP], ho[NP], gn2[NP], hn2[NP];
                    side_value_g<D, H, NPL>(L, cg, chh, gbuf, F.r.ownL, dO, A.dt, col, go, ho);
                    side_value_g<D, H, NPL>(L, cg, chh, gbuf, F.r.neiL, dN, A.dt, col, gn2, hn2);
#pragma unroll
                    for (int p = 0; p < NP; ++p) {
                        const float2 w = upwind_w2(xs[p]);
                        gf[p] = blend2(w, go[p], gn2[p]);
                        hf[p] = H ? blend2(w, ho[p], hn2[p]) : f2(0.f);
                    }
                } else if (D == 2 && F.plain == (3 | 3 << 8)) {  // two triangles
                    recon_plain32<D, H, NPL, 3>(A, tm.E, F, L, cg, chh, lane, v0, xs, gf, hf);
                } else if (D == 2 && F.plain == (4 | 4 << 8)) {  // two quadrilaterals
                    recon_plain32<D, H, NPL, 4>(A, tm.E, F, L, cg, chh, lane, v0, xs, gf, hf);
                } else {
                    recon32<D, H, NPL, false>(A, tm.E, F, L, cg, chh, lane, v0, xs, gf, hf, gw, hw);
                }
                mom32<D, H, NPL, NS, true>(m, L, ur, gf, hf, nullptr);
                stp<NP>(A.gF + fi, gf);
                if (H) stp<NP>(A.hF + fi, hf);
            } else {  // one side in T
                const bool own = F.r.ownL < hd.nT;
                const int nPlain = own ? F.plain & 255 : (F.plain >> 8) & 255;
                const int e0 = own ? F.r.stO0 : F.r.stN0, lu = own ? F.r.ownL : F.r.neiL;
                const float* du = own ? dO : dN;
                if (GR)
                    side_value_g<D, H, NPL>(L, cg, chh, gbuf, lu, du, A.dt, col, gf, hf);
                else if (D == 2 && nPlain == 3)
                    recon_one_plain32<D, H, NPL, 3>(A, tm.E, e0, lu, du[0], du[1], du[2], L, cg, chh, lane, v0, gf, hf);
                else if (D == 2 && nPlain == 4)
                    recon_one_plain32<D, H, NPL, 4>(A, tm.E, e0, lu, du[0], du[1], du[2], L, cg, chh, lane, v0, gf, hf);
                else
                    recon_one32<D, H, NPL>(A, tm.E, e0, own ? F.r.stO1 : F.r.stN1, lu, du[0], du[1], du[2], L, cg, chh,
                                           lane, v0, gf, hf);
                float2 wt[NP];
                float* dg = A.gF + fi;
                float* dh = H ? A.hF + fi : nullptr;
#pragma unroll
                for (int p = 0; p < NP; ++p) {
                    const float2 w = upwind_w2(xs[p]);
                    wt[p] = own ? w : sub2(f2(1.f), w);  // this side's share: 1 upwind, 1/2 tie
                    const bool u0 = wt[p].x == 1.f, u1 = wt[p].y == 1.f;
                    if (u0) {
                        dg[2 * p] = gf[p].x;
                        if (H) dh[2 * p] = hf[p].x;
                    }
                    if (u1) {
                        dg[2 * p + 1] = gf[p].y;
                        if (H) dh[2 * p + 1] = hf[p].y;
                    }
                }
                mom32<D, H, NPL, NS, true>(m, L, ur, gf, hf, wt);
            }
            const float tot = reduce_scatter<NS, float, SL::FLUX + 1>(m, lane);
            if (writer && myslot <= SL::FLUX) mom[lf * NS + myslot].add(tot);
        }
    }
    __syncthreads();
    // ---- per-side totals (FP64) to faceMom[a][side]
    for (int lf = threadIdx.x; lf < hd.nFB; lf += NW * 32) {
        const int4 rr = tm.F[5 * lf];  // {ownL, neiL, a, w}
        const bool own = rr.x < hd.nT, complete = rr.w >= 0 || (own && rr.y < hd.nT);
        double* dst = A.faceMom + (size_t)rr.z * 2 * NS;
        double* mine = dst + (own ? 0 : NS);
        for (int s = 0; s < NS; ++s) mine[s] = mom[lf * NS + s].value();
        if (complete)
            for (int s = 0; s < NS; ++s) dst[NS + s] = 0.0;
    }
}

template <int D, bool H, int NPL, int NW, bool GR>
__global__ void __launch_bounds__(NW * 32, 1) k_face_sides32(FusedArgs<float> A) {
    extern __shared__ __align__(16) unsigned char smem[];
    face_sides_body<D, H, NPL, NW, GR>(A, blockIdx.x, smem);
}

// Several independent cases in one launch: block b runs tile work[b].y of
// case work[b].x.  The cases' arguments are read through a read-only
// pointer; every case shares D, H and NPL.
template <int D, bool H, int NPL, int NW>
__global__ void __launch_bounds__(NW * 32, 1) k_face_sides32_batch(const FusedArgs<float>* __restrict__ AA,
                                                                   const int2* __restrict__ work) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ FusedArgs<float> sA;
    const int2 w = work[blockIdx.x];
    {
        const long long* src = reinterpret_cast<const long long*>(AA + w.x);
        long long* dst = reinterpret_cast<long long*>(&sA);
        for (int k = threadIdx.x; k < (int)(sizeof(FusedArgs<float>) / 8); k += blockDim.x) dst[k] = src[k];
    }
    __syncthreads();
    face_sides_body<D, H, NPL, NW, false>(sA, w.y, smem);
}

// Open boundary faces (zeroGradient, fixedValue -> mixed, farField, pressureIn,
// pressureOut), one warp per face, after sweep A stored their owner-side
// reconstruction for every velocity: the complete face values (deviation
// form) and their moments over all velocities, so that the face macros take
// the internal-face path.  zeroGradient: every velocity takes the owner's
// gbar+ (discreteVelocity.C:551-555); the others keep the outgoing
// reconstruction and set the incoming velocities (xi.S <= 0) to
// rho_b M(U of the owner cell, T_b) (:570-600) -- fixedValue to the
// Maxwellian of its patch rho, U, T, which stays as it was at the start
// (:302-345).  Symmetry faces (symmetryMod, symmetryPlane): the incoming
// velocities (xi.S0 <= 0, S0 the patch's first face) take their mirror
// velocity's value (discreteVelocity.C:733-817), read from a snapshot of the
// face row; symmetryPlane assigns in index order, so a mirror that is itself
// an earlier incoming velocity passes its own mirror's value on (the chain
// ends after one step on grids symmetric about 0).  A separate kernel keeps
// the sweep's code unchanged.
template <int D, bool H, int NPL>
__global__ void k_open_faces32(FusedArgs<float> A) {
    using SL = Slots<D, H>;
    constexpr int NS = SL::NS, KC = 32 * NPL, NP = NPL / 2;
    const StepArgs& b = A.b;
    const int lane = threadIdx.x & 31, Vp = b.Vp, col = lane * NPL;
    const int myslot = slot_of<NS>(lane);
    const bool writer = NS == 16 ? (lane & 1) == 0 : true;
    for (int w = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); w < b.nW; w += gridDim.x * (blockDim.x >> 5)) {
        const int kind = b.bKind[w];
        if (kind == kBcMaxwell) continue;  // warp-uniform
        const int a = b.nI + w, own = chk(b.own[a], b.nC, b.status);
        const float sx = (float)b.Sf[3 * a], sy = (float)b.Sf[3 * a + 1], sz = (float)b.Sf[3 * a + 2];
        const float4 u4 = A.uref4[a];
        const float ur[3] = {u4.x, u4.y, u4.z};
        Eq32<D, H> ec;
        float ng = 0.f, i2 = 0.f, hw = 0.f, ux = 0.f, uy = 0.f, uz = 0.f;
        const bool sym = kind == kBcSymmetryMod || kind == kBcSymmetryPlane;
        const double* S0 = b.bS0 + 3 * w;
        auto incoming = [&](int u) {
            return b.xi[u] * S0[0] + b.xi[Vp + u] * S0[1] + b.xi[2 * Vp + u] * S0[2] <= 0;
        };
        if (sym) {  // snapshot of the row
            const size_t fb = (size_t)a * Vp, wb = (size_t)w * Vp;
            for (int v = lane; v < Vp; v += 32) {
                A.symG[wb + v] = A.gF[fb + v];
                if (H) A.symH[wb + v] = A.hF[fb + v];
            }
            __syncwarp();
        } else if (kind == kBcZeroGradient) {
            const float* cblk = A.cc + (size_t)own * kNCoef;
            float4 q[3];
            eq_table(q, cblk, cell_weight(A.dt, cblk));
            ec.load(q, b.K, A.hrefFac);
        } else {
            const double Tb = b.TbM[w], RT = b.R * Tb;
            const double* U = kind == kBcFixedValue ? b.Uw + 3 * w : b.U + 3 * own;
            const double sq = sqrt(2.0 * kPi * RT);
            ng = (float)(A.gscale * b.rhoB[w] / (D == 2 ? sq * sq : sq * sq * sq));
            i2 = (float)(-0.5 / RT);
            hw = (float)(RT * (b.K + 3 - D));
            ux = (float)U[0]; uy = (float)U[1]; uz = (float)U[2];
        }
        Acc<float> acc;
        acc.zero();
        for (int v0 = 0; v0 < Vp; v0 += KC) {
            Lane32<D, NPL> L;
            L.load(A, v0, lane);
            const size_t fi = (size_t)a * Vp + v0 + col;
            float2 gf[NP], hf[NP];
            if (sym) {
                ldp<NP>(gf, A.gF + fi);
                if (H) ldp<NP>(hf, A.hF + fi);
                float* gs = reinterpret_cast<float*>(gf);
                float* hs = reinterpret_cast<float*>(hf);
                const int* tab = b.symTab + (size_t)b.symOff[w] * b.nV;
                const float* snG = A.symG + (size_t)w * Vp;
                const float* snH = H ? A.symH + (size_t)w * Vp : nullptr;
#pragma unroll
                for (int j = 0; j < NPL; ++j) {
                    const int v = v0 + col + j;
                    if (v >= b.nV || !incoming(v)) continue;
                    int cur = v, u = chk(tab[v], b.nV, b.status);
                    if (kind == kBcSymmetryPlane)
                        for (int guard = 0; guard < b.nV && u < cur && incoming(u); ++guard) {
                            cur = u;
                            u = chk(tab[u], b.nV, b.status);
                        }
                    gs[j] = snG[u];
                    if (H) hs[j] = snH[u];
                }
                if (!H)
#pragma unroll
                    for (int p = 0; p < NP; ++p) hf[p] = f2(0.f);
            } else if (kind == kBcZeroGradient) {
                const size_t ci = (size_t)own * Vp + v0 + col;
                ldp<NP>(gf, A.gT + ci);
                if (H) ldp<NP>(hf, A.hT + ci);
#pragma unroll
                for (int p = 0; p < NP; ++p) {
                    if (!H) hf[p] = f2(0.f);
                    ec.relax(L, p, gf[p], hf[p]);
                }
            } else {
                ldp<NP>(gf, A.gF + fi);
                if (H) ldp<NP>(hf, A.hF + fi);
#pragma unroll
                for (int p = 0; p < NP; ++p) {
                    float2 xs = fma2(L.y[p], f2(sy), mul2(L.x[p], f2(sx)));
                    if (D == 3) xs = fma2(L.z[p], f2(sz), xs);
                    const float2 cx = sub2(L.x[p], f2(ux)), cy = sub2(L.y[p], f2(uy));
                    float2 cc = fma2(cy, cy, mul2(cx, cx));
                    if (D == 3) {
                        const float2 cz = sub2(L.z[p], f2(uz));
                        cc = fma2(cz, cz, cc);
                    }
                    const float2 m = make_float2(ng * expf(i2 * cc.x), ng * expf(i2 * cc.y));
                    const bool o0 = xs.x > 0.f, o1 = xs.y > 0.f;
                    gf[p] = sel2(o0, o1, gf[p], sub2(m, L.mr[p]));
                    if (H) hf[p] = sel2(o0, o1, hf[p], sub2(mul2(m, f2(hw)), mul2(L.mr[p], f2(A.hrefFac))));
                }
            }
            stp<NP>(A.gF + fi, gf);
            if (H) stp<NP>(A.hF + fi, hf);
            float m[NS];
#pragma unroll
            for (int s2 = 0; s2 < NS; ++s2) m[s2] = 0.0f;
            mom32<D, H, NPL, NS>(m, L, ur, gf, hf, nullptr);
            acc.add(reduce_scatter<NS, float, SL::FLUX + 1>(m, lane));
        }
        double* dst = A.faceMom + (size_t)a * 2 * NS;
        if (writer && myslot < NS) {
            dst[myslot] = myslot < SL::FLUX ? acc.value() : 0.0;
            dst[NS + myslot] = 0.0;
        }
    }
}

// Face macros of every active face from the two per-side moment totals.
template <int D, bool H>
__device__ __forceinline__ void face_macros_one(const FusedArgs<float>& A, int a) {
    constexpr int NS = Slots<D, H>::NS;
    const double* src = A.faceMom + (size_t)a * 2 * NS;
    double M[NS];
    for (int s = 0; s < NS; ++s) M[s] = src[s] + src[NS + s];
    const int w = a >= A.b.nI && A.b.bKind[a - A.b.nI] == kBcMaxwell ? a - A.b.nI : -1;
    finalize_face32<D, H>(A, a, w, A.uref4[a], M);
}

template <int D, bool H>
__global__ void k_face_macros32(FusedArgs<float> A) {
    for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < A.b.nA; a += gridDim.x * blockDim.x)
        face_macros_one<D, H>(A, a);
}

// Case of a global item index: off[] holds the first item of each case (n+1 entries).
__device__ __forceinline__ int case_of(const int* __restrict__ off, int n, int g) {
    int lo = 0, hi = n;  // off[lo] <= g < off[hi]
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (off[mid] <= g) lo = mid;
        else hi = mid;
    }
    return lo;
}

template <int D, bool H>
__global__ void k_face_macros32_batch(const FusedArgs<float>* __restrict__ AA, const int* __restrict__ faceOff,
                                      int nCases) {
    const int total = faceOff[nCases];
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < total; g += gridDim.x * blockDim.x) {
        const int i = case_of(faceOff, nCases, g);
        face_macros_one<D, H>(AA[i], g - faceOff[i]);
    }
}

// ---------------------------------------------------------------- sweep B, gather form
// Shared memory of the gather sweep: per warp two stages of (1 + MF) rows of
// g (and h): the cell's g~ row and its first MF faces' stored values.
__host__ __device__ inline size_t gather_smem(int nw, int mf, int kc, bool h) {
    return (size_t)nw * 2 * (1 + mf) * (h ? 2 : 1) * kc * sizeof(float);
}

// Cell macros (FP64) from the deviation moment totals M (slots as Slots<D,H>).
template <int D, bool H, typename TT = double>
__device__ __forceinline__ void finalize_cell32(const FusedArgs<float>& A, int c, const TT* tot) {
    using SL = Slots<D, H>;
    constexpr int NS = SL::NS;
    const StepArgs& b = A.b;
    const float4 u4 = reinterpret_cast<const float4*>(A.cc + (size_t)c * kNCoef)[0];
    const double ur[3] = {u4.x, u4.y, u4.z};
    double M[NS], Rm[NS];
    ref_moments_about<D, H>(A.refMom, ur, Rm);
    for (int s = 0; s < SL::NM; ++s) M[s] = (tot[s] + Rm[s]) * A.invGscale;
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

// Cells per warp batch of the gather sweep's FP64 macro step (one lane per cell).
constexpr int kGatherBatch = 32;

// One cell of the gather sweep, all DV chunks; returns this lane's slot total
// of the new cell moments (slot slot_of(lane)).  wb: the warp's two stages,
// offset by the lane's column.
// OPEN: the case has open boundary faces (instantiated apart so that
// wall-only cases run the same code as before those existed).
// tab: the velocity constants in shared memory (dv_table32), or null.
template <int D, bool H, int NPL, bool OPEN = false>
__device__ __forceinline__ double gather_cell(const FusedArgs<float>& A, int c, int MF, float* wb, int lane,
                                              const float* tab = nullptr) {
    using SL = Slots<D, H>;
    constexpr int NS = SL::NS, KC = 32 * NPL, NP = NPL / 2, NR = H ? 2 : 1;
    const StepArgs& b = A.b;
    const int Vp = b.Vp, col = lane * NPL;
    const int stageRows = (1 + MF) * NR;
    const int e0 = A.cfOff[c], e1 = A.cfOff[c + 1];
    const int nfs = min(e1 - e0, MF);  // faces staged through shared memory
    auto issue = [&](int stage, int v0) {
        float* st = wb + (size_t)stage * stageRows * KC;
        const size_t gi = (size_t)c * Vp + v0 + col;
        cp_async_row(st, A.gT + gi, NPL);
        if (H) cp_async_row(st + KC, A.hT + gi, NPL);
        for (int f = 0; f < nfs; ++f) {
            const int a = chk(__float_as_int(A.cfEnt[e0 + f].w), b.nA, b.status);
            const size_t fi = (size_t)a * Vp + v0 + col;
            cp_async_row(st + (1 + f) * NR * KC, A.gF + fi, NPL);
            if (H) cp_async_row(st + ((1 + f) * NR + 1) * KC, A.hF + fi, NPL);
        }
        cp_async_commit();
    };
    const float* cblk = A.cc + (size_t)c * kNCoef;
    Eq32<D, H> ec;
    {
        float4 q[3];
        eq_table(q, cblk, cell_weight(A.dt, cblk));
        ec.load(q, b.K, A.hrefFac);
    }
    const float4 u4 = reinterpret_cast<const float4*>(cblk)[0];
    const float ur[3] = {u4.x, u4.y, u4.z};
    const float kv = -A.dt * A.invVf[c];
    // cell moments: per-lane partial sums over all chunks, one warp reduction per cell
    float m[NS];
#pragma unroll
    for (int s2 = 0; s2 < NS; ++s2) m[s2] = 0.0f;
    const int nChunks = Vp / KC;
    issue(0, 0);
    for (int ch = 0; ch < nChunks; ++ch) {
        const int v0 = ch * KC;
        if (ch + 1 < nChunks) {
            issue((ch + 1) & 1, v0 + KC);
            cp_async_wait<1>();
        } else {
            cp_async_wait<0>();
        }
        const float* st = wb + (size_t)(ch & 1) * stageRows * KC;
        Lane32<D, NPL> L;
        if (tab) L.load_tab(tab, Vp, v0, lane);
        else L.load(A, v0, lane);
        float2 g0[NP], h0[NP], t[NP], th[NP];
        ldp<NP>(g0, st);
        if (H) ldp<NP>(h0, st + KC);
#pragma unroll
        for (int p = 0; p < NP; ++p) {
            float2 g = g0[p], h = H ? h0[p] : f2(0.f);
            ec.relax(L, p, g, h);
            t[p] = fma2(sub2(g, g0[p]), f2(1.0f / 3.0f), g);  // exact when g+ == g~
            th[p] = H ? fma2(sub2(h, h0[p]), f2(1.0f / 3.0f), h) : f2(0.f);
        }
#pragma unroll 3  // a triangle's three faces: independent relaxations interleave
        for (int e = e0; e < e1; ++e) {
            const int f = e - e0;
            const float4 ent = A.cfEnt[e];
            const int a = chk(__float_as_int(ent.w), b.nA, b.status);
            float2 gf[NP], hf[NP];
            if (f < nfs) {
                ldp<NP>(gf, st + (1 + f) * NR * KC);
                if (H) ldp<NP>(hf, st + ((1 + f) * NR + 1) * KC);
            } else {
                const size_t fi = (size_t)a * Vp + v0 + col;
                ldp<NP>(gf, A.gF + fi);
                if (H) ldp<NP>(hf, A.hF + fi);
            }
            if (!H)
#pragma unroll
                for (int p = 0; p < NP; ++p) hf[p] = f2(0.f);
            Eq32<D, H> eq;
            eq.load(A.feqT + 3 * (size_t)a, b.K, A.hrefFac);
            float2 xs[NP];
#pragma unroll
            for (int p = 0; p < NP; ++p) {
                xs[p] = fma2(L.y[p], f2(ent.y), mul2(L.x[p], f2(ent.x)));
                if (D == 3) xs[p] = fma2(L.z[p], f2(ent.z), xs[p]);
            }
            if (a >= b.nI) {  // boundary: the cell is the owner; outgoing where xi.S > 0
                const int w = a - b.nI;
                const float4 w4 = A.wall4[w];
                if (OPEN && w4.z != 0.f) {  // open boundary: incoming stored, unrelaxed
                    const bool plane = w4.z == 2.f;  // symmetryPlane: every DV once, outgoing twice
#pragma unroll
                    for (int p = 0; p < NP; ++p) {
                        if (plane) eq.relax(L, p, gf[p], hf[p]);
                        float2 go = gf[p], ho = hf[p];
                        eq.relax(L, p, go, ho);
                        const bool o0 = xs[p].x > 0.f, o1 = xs[p].y > 0.f;
                        gf[p] = sel2(o0, o1, go, gf[p]);
                        if (H) hf[p] = sel2(o0, o1, ho, hf[p]);
                    }
                } else {  // diffuse wall: incoming rho_w Mw
                    const float rws = A.rhoWs[w], hwf = w4.x;
                    float2 mw[NP];
                    ldp<NP>(mw, A.Mw + (size_t)w * Vp + v0 + col);
#pragma unroll
                    for (int p = 0; p < NP; ++p) {
                        float2 go = gf[p], ho = hf[p];
                        eq.relax(L, p, go, ho);
                        const float2 gw = mul2(f2(rws), mw[p]);
                        const bool o0 = xs[p].x > 0.f, o1 = xs[p].y > 0.f;
                        gf[p] = sel2(o0, o1, go, sub2(gw, L.mr[p]));
                        if (H) hf[p] = sel2(o0, o1, ho, sub2(mul2(gw, f2(hwf)), mul2(L.mr[p], f2(A.hrefFac))));
                    }
                }
            } else {
#pragma unroll
                for (int p = 0; p < NP; ++p) eq.relax(L, p, gf[p], hf[p]);
            }
#pragma unroll
            for (int p = 0; p < NP; ++p) {
                const float2 kx = mul2(xs[p], f2(kv));
                t[p] = fma2(kx, gf[p], t[p]);
                if (H) th[p] = fma2(kx, hf[p], th[p]);
            }
        }
        const size_t gi = (size_t)c * Vp + v0 + col;
        stp_cs<NP>(A.gTn + gi, t);
        if (H) stp_cs<NP>(A.hTn + gi, th);
        mom32<D, H, NPL, NS>(m, L, ur, t, th, nullptr);
    }
    return (double)reduce_scatter<NS, float, SL::NM>(m, lane);
}

// Warps stride over the cells (persistent grid); per cell, all DV chunks:
//   g~new = g+ + (g+ - g~)/3 - dt/V sum_f (xi.S_f) g^f_f,
// with g+ the cell relaxation of g~ (P1), g^f_f the face value stored by
// sweep A relaxed toward the face equilibrium (P7; incoming wall DVs take
// rho_w Mw unrelaxed) and the sum over the cell's faces in face order (P8),
// then the cell moments (P9).  Faces are relaxed once from each side; no
// tiles or block barriers.  The rows of chunk k+1 are copied into the warp's
// other stage while chunk k is computed; the FP64 macros of a batch of cells
// are finished together, one lane per cell.
// dvTab: the launch gave room after the stages for the velocity constants
// (dv_table32), read from there per chunk instead of from global memory.
// The batch of warp totals is kept in FP32: each total is an FP32 warp sum.
template <int D, bool H, int NPL, int NW, bool OPEN = false>
__global__ void __launch_bounds__(NW * 32, 2) k_cell_gather32(FusedArgs<float> A, int MF, int dvTab) {
    constexpr int NS = Slots<D, H>::NS, KC = 32 * NPL, NR = H ? 2 : 1;
    // 3D: half the batch -- the finalize is a small share of a 63-chunk cell,
    // and the smaller buffer leaves the L1 more room (8.40 -> 8.21 ms, 48^3 hexes)
    constexpr int GB = D == 3 ? kGatherBatch / 2 : kGatherBatch;
    __shared__ float sM[NW][GB][NS];
    __shared__ int sC[NW][GB];
    extern __shared__ __align__(16) float gsm[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    float* wb = gsm + (size_t)warp * 2 * (1 + MF) * NR * KC + lane * NPL;
    float* tab = nullptr;
    if (dvTab) {
        tab = gsm + gather_smem(NW, MF, KC, H) / sizeof(float);
        dv_table32<D>(A, tab);
        __syncthreads();
    }
    const int myslot = slot_of<NS>(lane);
    const bool writer = NS == 16 ? (lane & 1) == 0 : true;
    const int TW = gridDim.x * NW, nC = A.b.nC;
    int nb = 0;
    for (int c = blockIdx.x * NW + warp; c < nC; c += TW) {
        const double tot = gather_cell<D, H, NPL, OPEN>(A, c, MF, wb, lane, tab);
        if (writer) sM[warp][nb][myslot] = (float)tot;
        if (lane == 0) sC[warp][nb] = c;
        ++nb;
        if (nb == GB || c + TW >= nC) {
            __syncwarp();
            if (lane < nb) finalize_cell32<D, H>(A, sC[warp][lane], sM[warp][lane]);
            __syncwarp();
            nb = 0;
        }
    }
}

// Several independent cases in one launch: warps stride over the cells of
// all cases (cellOff: first global cell of each case, nCases+1 entries).
template <int D, bool H, int NPL, int NW>
__global__ void __launch_bounds__(NW * 32, 2) k_cell_gather32_batch(const FusedArgs<float>* __restrict__ AA,
                                                                    const int* __restrict__ cellOff, int nCases, int MF) {
    constexpr int NS = Slots<D, H>::NS, KC = 32 * NPL, NR = H ? 2 : 1;
    __shared__ float sM[NW][kGatherBatch][NS];  // FP32 warp totals, exact
    __shared__ int sC[NW][kGatherBatch], sI[NW][kGatherBatch];
    __shared__ FusedArgs<float> sA[NW];  // the warp's current case
    extern __shared__ __align__(16) float gsm[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    float* wb = gsm + (size_t)warp * 2 * (1 + MF) * NR * KC + lane * NPL;
    const int myslot = slot_of<NS>(lane);
    const bool writer = NS == 16 ? (lane & 1) == 0 : true;
    const int TW = gridDim.x * NW, total = cellOff[nCases];
    int nb = 0, cur = -1;
    for (int g = blockIdx.x * NW + warp; g < total; g += TW) {
        const int i = case_of(cellOff, nCases, g), c = g - cellOff[i];
        if (i != cur) {  // consecutive cells mostly share a case: copy its arguments once
            static_assert(sizeof(FusedArgs<float>) % 8 == 0, "argument block is copied in 8-byte words");
            const long long* src = reinterpret_cast<const long long*>(AA + i);
            long long* dst = reinterpret_cast<long long*>(&sA[warp]);
            __syncwarp();
            for (int k = lane; k < (int)(sizeof(FusedArgs<float>) / 8); k += 32) dst[k] = src[k];
            __syncwarp();
            cur = i;
        }
        const double tot = gather_cell<D, H, NPL>(sA[warp], c, MF, wb, lane);
        if (writer) sM[warp][nb][myslot] = (float)tot;
        if (lane == 0) { sC[warp][nb] = c; sI[warp][nb] = i; }
        ++nb;
        if (nb == kGatherBatch || g + TW >= total) {
            __syncwarp();
            if (lane < nb) finalize_cell32<D, H>(AA[sI[warp][lane]], sC[warp][lane], sM[warp][lane]);
            __syncwarp();
            nb = 0;
        }
    }
}

// ------------------------------------------------- persistent batched step
// Grid-wide barrier of a cooperative launch (every block resident): an
// arrival counter bar[0] and a generation bar[1] in global memory (zeroed
// before the launch).  Arrival is an acquire-release add, the last arrival
// releases the generation and the waiters acquire it, so that after the
// barrier every block sees what every block wrote before it (the acquire
// also keeps stale L1 lines from being read).  A wait polls at most `cap`
// times; then it sets *status = DUGKS_ERR_TIMEOUT (6) and the barrier returns
// false in every block that reaches it afterwards, so all blocks leave the
// kernel.  Callers reach it only with no asynchronous copy in flight.
constexpr int kStatusTimeout = 6;
__device__ __forceinline__ bool grid_barrier(unsigned* bar, long long cap, int* status) {
    __shared__ int sOk;
    __syncthreads();
    if (threadIdx.x == 0) {
        int ok = 1;
        const unsigned gen = *(volatile unsigned*)(bar + 1);
        unsigned old;
        asm volatile("atom.add.acq_rel.gpu.global.u32 %0, [%1], 1;" : "=r"(old) : "l"(bar) : "memory");
        if (old == gridDim.x - 1) {  // last to arrive: reset, release the others
            atomicExch(bar, 0u);
            asm volatile("red.release.gpu.global.add.u32 [%0], 1;" ::"l"(bar + 1) : "memory");
        } else {
            long long it = 0;
            for (;;) {
                unsigned g;
                asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(g) : "l"(bar + 1) : "memory");
                if (g != gen) break;
                if (++it > cap) {
                    ok = 0;
                    atomicExch(status, kStatusTimeout);
                    break;
                }
                __nanosleep(64);
            }
        }
        if (*(volatile int*)status == kStatusTimeout) ok = 0;
        sOk = ok;
    }
    __syncthreads();
    return sOk != 0;
}

// Cells finished per warp batch in the persistent kernel's gather pass.
constexpr int kPersistBatch = 16;

// Dynamic shared memory of the persistent kernel's gather pass: the warps'
// row stages, their case-argument copies, slot totals and cell / case ids.
template <int D, bool H>
__host__ __device__ inline size_t persist_gather_smem(int nw, int mf, int kc) {
    return gather_smem(nw, mf, kc, H) + (size_t)nw * sizeof(FusedArgs<float>) +
           (size_t)nw * kPersistBatch * Slots<D, H>::NS * sizeof(double) + 2 * (size_t)nw * kPersistBatch * sizeof(int);
}

// Several independent cases, nSteps whole steps in one cooperative launch:
// per step the face-side tiles of all cases (blocks stride over the work
// list), a grid barrier, the face macros of all cases (threads stride over
// the faces), a barrier, the cell gather of all cases (warps stride over the
// cells), a barrier.  Step s uses the argument arrays of parity
// (parity0 + s) & 1 (double buffers swapped).  The pass bodies are those of
// the single-case kernels.
template <int D, bool H, int NPL, int NW>
__global__ void __launch_bounds__(NW * 32, 1)
    k_batch_persistent32(const FusedArgs<float>* __restrict__ AA0, const FusedArgs<float>* __restrict__ AA1,
                         const int2* __restrict__ work, int nWork, const int* __restrict__ faceOff,
                         const int* __restrict__ cellOff, int nCases, int MF, int nSteps, int parity0, unsigned* bar,
                         long long cap, int* status) {
    using SL = Slots<D, H>;
    constexpr int NS = SL::NS, KC = 32 * NPL, NR = H ? 2 : 1;
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ FusedArgs<float> sA;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    constexpr int W8 = (int)(sizeof(FusedArgs<float>) / 8);
    static_assert(sizeof(FusedArgs<float>) % 8 == 0, "argument block is copied in 8-byte words");
    // gather-pass carve-up of the dynamic shared memory
    float* gsm = reinterpret_cast<float*>(smem);
    const size_t stBytes = gather_smem(NW, MF, KC, H);
    FusedArgs<float>* sAw = reinterpret_cast<FusedArgs<float>*>(smem + stBytes);
    double* sM = reinterpret_cast<double*>(smem + stBytes + NW * sizeof(FusedArgs<float>));
    int* sC = reinterpret_cast<int*>(sM + (size_t)NW * kPersistBatch * NS);
    int* sI = sC + NW * kPersistBatch;
    float* wb = gsm + (size_t)warp * 2 * (1 + MF) * NR * KC + lane * NPL;
    const int myslot = slot_of<NS>(lane);
    const bool writer = NS == 16 ? (lane & 1) == 0 : true;
    const int totalFaces = faceOff[nCases], totalCells = cellOff[nCases];
    for (int s = 0; s < nSteps; ++s) {
        const FusedArgs<float>* AA = ((parity0 + s) & 1) ? AA1 : AA0;
        // ---- face sides (P1-P3 and the per-side face moments)
        for (int w = blockIdx.x; w < nWork; w += gridDim.x) {
            const int2 wk = work[w];
            const long long* src = reinterpret_cast<const long long*>(AA + wk.x);
            long long* dst = reinterpret_cast<long long*>(&sA);
            for (int k = threadIdx.x; k < W8; k += blockDim.x) dst[k] = src[k];
            __syncthreads();
            face_sides_body<D, H, NPL, NW, false>(sA, wk.y, smem);
            __syncthreads();
        }
        if (!grid_barrier(bar, cap, status)) return;
        // ---- face macros (P4-P6)
        for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < totalFaces; g += gridDim.x * blockDim.x) {
            const int i = case_of(faceOff, nCases, g);
            face_macros_one<D, H>(AA[i], g - faceOff[i]);
        }
        if (!grid_barrier(bar, cap, status)) return;
        // ---- cell gather (P7-P9)
        int nb = 0, cur = -1;
        const int TW = gridDim.x * NW;
        for (int g = blockIdx.x * NW + warp; g < totalCells; g += TW) {
            const int i = case_of(cellOff, nCases, g), c = g - cellOff[i];
            if (i != cur) {
                const long long* src = reinterpret_cast<const long long*>(AA + i);
                long long* dst = reinterpret_cast<long long*>(sAw + warp);
                __syncwarp();
                for (int k = lane; k < W8; k += 32) dst[k] = src[k];
                __syncwarp();
                cur = i;
            }
            const double tot = gather_cell<D, H, NPL>(sAw[warp], c, MF, wb, lane);
            double* mw = sM + ((size_t)warp * kPersistBatch + nb) * NS;
            if (writer) mw[myslot] = tot;
            if (lane == 0) { sC[warp * kPersistBatch + nb] = c; sI[warp * kPersistBatch + nb] = i; }
            ++nb;
            if (nb == kPersistBatch || g + TW >= totalCells) {
                __syncwarp();
                if (lane < nb)
                    finalize_cell32<D, H>(AA[sI[warp * kPersistBatch + lane]], sC[warp * kPersistBatch + lane],
                                          sM + ((size_t)warp * kPersistBatch + lane) * NS);
                __syncwarp();
                nb = 0;
            }
        }
        if (!grid_barrier(bar, cap, status)) return;
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
