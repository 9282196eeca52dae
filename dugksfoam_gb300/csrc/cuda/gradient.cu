// Differentiated FP64 step: tangent-linear (forward mode, Dual numbers) and
// hand-written adjoint (reverse mode) of the reference-pipeline step
// (ref_pipeline.cu, i.e. fvDVM::evolution, src/fvDVM/fvDVM/fvDVM.C:1086-1108),
// with respect to the wall temperatures T_w (per wall face) and the viscosity
// scale mu_ref (tau = mu_ref (T/Tref)^omega / (rho R T), fvDVM::updateTau,
// fvDVM.C:808-817).  Objective: sum over a window of steps of
//   sum_w S_w . qWall_w  (one patch)  +  sum_w |S_w| stressWall_w,xy  (one patch),
// with qWall / stressWall as fvDVM::updateMacroSurf forms them (fvDVM.C:535-576).
//
// Tangent-linear kernels (t_*) are the reference-pipeline kernels with the
// state carried as Dual (value, derivative along one parameter direction).
// Adjoint kernels (r_*) run the passes in reverse:
//   r_cell_mom  P9  cell macros        <- g~n+1
//   r_cell_flux P8  g~n+1 = -g~/3 + 4/3 gbar+ - dt/V sum (xi.S) g_f
//   r_face      P7  face relaxation, P6 face macros (+ objective seeds)
//   r_wall      P5  incoming rho_w M_w, P4 rho_w = outgoing / |inComingByRho(T_w)|
//   r_recon     P3  upwind reconstruction (+ lagged wall gradient output)
//   r_grad      P2  least-squares gradient (+ lagged wall gradient input)
//   r_barp      P1  cell relaxation toward the Shakhov equilibrium
// Local Jacobians are analytic (Shakhov and Maxwellian in (rho, U, T, q)).
#include "device_common.cuh"
#include "dual.cuh"
#include "gradient.h"

namespace dugks {
namespace {

constexpr int kT = 256;
constexpr int kRT = 128;

int grid(long long n, int threads, int sms) {
    long long b = (n + threads - 1) / threads;
    long long cap = (long long)sms * 32;
    return (int)(b < cap ? (b > 0 ? b : 1) : cap);
}

__device__ __forceinline__ void dvi(long long i, int Vp, int& e, int& v) {
    e = (int)(i / Vp);
    v = (int)(i - (long long)e * Vp);
}

// ------------------------------------------------------------ shared forms
template <class R>
__device__ __forceinline__ void shakhovT(R rho, R Ux, R Uy, R Uz, R T, R qx, R qy, R qz, double xx, double xy,
                                         double xz, double Rg, double Pr, int D, int K, R& gEq, R& hEq) {
    R ax = Ux - xx, ay = Uy - xy, az = Uz - xz;
    R cSqrByRT = (ax * ax + ay * ay + az * az) / (Rg * T);
    R cq = ((xx - Ux) * qx + (xy - Uy) * qy + (xz - Uz) * qz) / (5.0 * rho * Rg * T * Rg * T);
    R s = sqrt(2.0 * kPi * Rg * T);
    R pw = (D == 2) ? s * s : (D == 3 ? s * s * s : s);
    R gB = rho / pw * exp(-cSqrByRT / 2.0);
    R pc = (1.0 - Pr) * cq;
    gEq = (1.0 + pc * (cSqrByRT - D - 2.0)) * gB;
    hEq = ((K + 3.0 - D) + pc * ((cSqrByRT - D) * (K + 3.0 - D) - 2 * K)) * gB * Rg * T;
}

template <class R>
__device__ __forceinline__ R maxwellT(double Ux, double Uy, double Uz, R T, double xx, double xy, double xz,
                                      double Rg, int D) {
    double ax = Ux - xx, ay = Uy - xy, az = Uz - xz;
    R s = sqrt(2.0 * kPi * Rg * T);
    R pw = (D == 2) ? s * s : (D == 3 ? s * s * s : s);
    return 1.0 / pw * exp(-(ax * ax + ay * ay + az * az) / (2.0 * Rg * T));
}

template <class R>
__device__ __forceinline__ R tauT(R T, R rho, R muRef, double omega, double Tref, double Rg) {
    return muRef * exp(omega * log(T / Tref)) / rho / T / Rg;
}

// Shakhov equilibrium and its partial derivatives with respect to
// m = (rho, Ux, Uy, Uz, T, qx, qy, qz).  With theta = R T, c = xi - U,
// a = |c|^2/theta, G0 = (2 pi theta)^(-D/2) exp(-a/2), kap = (1-Pr)/(5 theta^2):
//   gE = rho G0 + kap (c.q)(a - D - 2) G0
//   hE = theta [k3 rho G0 + kap (c.q) B G0],  k3 = K+3-D,  B = (a-D) k3 - 2K.
// The per-entity factors (1/theta, the normalisation, kap) are formed once
// (ShakhovJac::prep); each velocity then costs one exp and products.
struct ShakhovJac {
    double rho, U[3], q[3], th, ith, N, kap, R, k3, K2;
    int D;
    __device__ __forceinline__ void prep(const double* m, double Rg, double Pr, int Dd, int K) {
        rho = m[0];
        for (int k = 0; k < 3; ++k) { U[k] = m[1 + k]; q[k] = m[5 + k]; }
        th = Rg * m[4];
        ith = 1.0 / th;
        const double s = sqrt(2.0 * kPi * th);
        N = 1.0 / ((Dd == 2) ? s * s : (Dd == 3 ? s * s * s : s));
        kap = (1.0 - Pr) / 5.0 * ith * ith;
        R = Rg;
        D = Dd;
        k3 = K + 3.0 - Dd;
        K2 = 2.0 * K;
    }
    __device__ __forceinline__ void eval(double x0, double x1, double x2, double& gE, double& hE, double* dg,
                                         double* dh) const {
        const double c[3] = {x0 - U[0], x1 - U[1], x2 - U[2]};
        const double a = (c[0] * c[0] + c[1] * c[1] + c[2] * c[2]) * ith;
        const double G0 = N * exp(-0.5 * a);
        const double cq = c[0] * q[0] + c[1] * q[1] + c[2] * q[2];
        const double B = (a - D) * k3 - K2, P = a - D - 2.0;
        const double kG = kap * G0, kGcq = kG * cq;
        gE = rho * G0 + kGcq * P;
        const double H = k3 * rho * G0 + kGcq * B;
        hE = th * H;
        dg[0] = G0;
        dh[0] = th * k3 * G0;
        // U_k: with ck = c_k / theta
        const double gU = rho * G0 + kGcq * (P - 2.0), hU = k3 * rho * G0 + kGcq * (B - 2.0 * k3);
        for (int k = 0; k < 3; ++k) {
            const double ck = c[k] * ith;
            dg[1 + k] = gU * ck - kG * q[k] * P;
            dh[1 + k] = hU * c[k] - th * kG * q[k] * B;
        }
        // T via theta: dG0/dtheta = G0 (a - D) / (2 theta)
        const double hd = 0.5 * (a - D) * ith;
        const double dgth = rho * G0 * hd + kGcq * ith * (-2.0 * P - a + P * (a - D) * 0.5);
        const double dHth = k3 * rho * G0 * hd + kGcq * ith * (-2.0 * B - k3 * a + B * (a - D) * 0.5);
        dg[4] = R * dgth;
        dh[4] = R * (H + th * dHth);
        for (int k = 0; k < 3; ++k) {
            dg[5 + k] = kG * c[k] * P;
            dh[5 + k] = th * kG * c[k] * B;
        }
    }
};

// ============================================================ tangent-linear
struct TArgs {
    StepArgs a;
    Dual *rho, *U, *T, *q, *tau;
    Dual *rhoF, *UF, *TF, *qF, *tauF;
    Dual *rhoW, *qWall, *stressWall;
    const Dual* Tw;
    Dual* incAbs;
    Dual muRef;
};

__global__ void t_incabs(TArgs t) {
    __shared__ double red[32 * 2];
    const StepArgs& a = t.a;
    const int wf = blockIdx.x, Vp = a.Vp;
    const double* S = a.Sf + 3 * (a.nI + wf);
    const double* Uw = a.Uw + 3 * wf;
    double acc[2] = {0.0, 0.0};
    for (int v = threadIdx.x; v < a.nV; v += blockDim.x) {
        double x0 = a.xi[v], x1 = a.xi[Vp + v], x2 = a.xi[2 * Vp + v];
        double xs = x0 * S[0] + x1 * S[1] + x2 * S[2];
        if (xs < 0) {
            Dual M = maxwellT<Dual>(Uw[0], Uw[1], Uw[2], t.Tw[wf], x0, x1, x2, a.R, a.D);
            Dual r = -a.w[v] * xs * M;
            acc[0] += r.v;
            acc[1] += r.d;
        }
    }
    block_sum<2>(acc, red);
    if (threadIdx.x == 0) t.incAbs[wf] = fabs(Dual{acc[0], acc[1]});
}

__global__ void t_init(TArgs t, const double* rho0, const double* U0, const double* T0, Dual* gT, Dual* hT) {
    const StepArgs& a = t.a;
    const long long n = (long long)a.nC * a.Vp;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        int c, v;
        dvi(i, a.Vp, c, v);
        if (v == 0) {
            t.rho[c] = dual(rho0[c]);
            for (int k = 0; k < 3; ++k) { t.U[3 * c + k] = dual(U0[3 * c + k]); t.q[3 * c + k] = dual(0.0); }
            t.T[c] = dual(T0[c]);
            t.tau[c] = tauT<Dual>(dual(T0[c]), dual(rho0[c]), t.muRef, a.omega, a.Tref, a.R);
        }
        if (v >= a.nV) { gT[i] = dual(0); if (a.hasH) hT[i] = dual(0); continue; }
        double ge, he;
        shakhov_ref(rho0[c], U0[3 * c], U0[3 * c + 1], U0[3 * c + 2], T0[c], 0.0, 0.0, 0.0, a.xi[v], a.xi[a.Vp + v],
                    a.xi[2 * a.Vp + v], a.R, a.Pr, a.D, a.K, ge, he);
        gT[i] = dual(ge);
        if (a.hasH) hT[i] = dual(he);
    }
}

__global__ void t_barp(TArgs t, const Dual* gT, const Dual* hT, Dual* gB, Dual* hB) {
    const StepArgs& a = t.a;
    const long long n = (long long)a.nC * a.Vp;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        int c, v;
        dvi(i, a.Vp, c, v);
        if (v >= a.nV) continue;
        const double dt = a.dt;
        Dual rf = 1.5 * dt / (2.0 * t.tau[c] + dt);
        Dual ge, he;
        shakhovT<Dual>(t.rho[c], t.U[3 * c], t.U[3 * c + 1], t.U[3 * c + 2], t.T[c], t.q[3 * c], t.q[3 * c + 1],
                       t.q[3 * c + 2], a.xi[v], a.xi[a.Vp + v], a.xi[2 * a.Vp + v], a.R, a.Pr, a.D, a.K, ge, he);
        gB[i] = (1.0 - rf) * gT[i] + rf * ge;
        if (a.hasH) hB[i] = (1.0 - rf) * hT[i] + rf * he;
    }
}

__global__ void t_grad(TArgs t, const Dual* gB, const Dual* hB, Dual* gG, Dual* hG, Dual* Gbg, Dual* Gbh) {
    const StepArgs& a = t.a;
    const long long n = (long long)a.nC * a.Vp;
    const int D = a.D, Vp = a.Vp;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        int c, v;
        dvi(i, Vp, c, v);
        if (v >= a.nV) continue;
        Dual g[3] = {dual(0), dual(0), dual(0)}, h[3] = {dual(0), dual(0), dual(0)};
        const Dual gc = gB[i];
        const Dual hc = a.hasH ? hB[i] : dual(0);
        for (int j = a.cellOff[c]; j < a.cellOff[c + 1]; ++j) {
            int e = a.cellFace[j], f = e >> 1, side = e & 1;
            if (f < a.nI) {
                int o = a.own[f], nb = a.nei[f];
                Dual dg = gB[(long long)nb * Vp + v] - gB[(long long)o * Vp + v];
                Dual dh = a.hasH ? hB[(long long)nb * Vp + v] - hB[(long long)o * Vp + v] : dual(0);
                const double* L = side ? a.nVec + 3 * f : a.pVec + 3 * f;
                if (side == 0) {
                    for (int k = 0; k < D; ++k) { g[k] += L[k] * dg; h[k] += L[k] * dh; }
                } else {
                    for (int k = 0; k < D; ++k) { g[k] -= L[k] * dg; h[k] -= L[k] * dh; }
                }
            } else {
                int wf = f - a.nI;
                long long wi = (long long)wf * Vp + v;
                Dual dg = (gc + Gbg[wi] / a.dcW[wf]) - gc;
                Dual dh = a.hasH ? (hc + Gbh[wi] / a.dcW[wf]) - hc : dual(0);
                const double* L = a.bVec + 3 * wf;
                for (int k = 0; k < D; ++k) { g[k] += L[k] * dg; h[k] += L[k] * dh; }
            }
        }
        for (int k = 0; k < D; ++k) {
            gG[((long long)c * D + k) * Vp + v] = g[k];
            if (a.hasH) hG[((long long)c * D + k) * Vp + v] = h[k];
        }
        for (int j = a.cellOff[c]; j < a.cellOff[c + 1]; ++j) {
            int f = a.cellFace[j] >> 1;
            if (f < a.nI) continue;
            int wf = f - a.nI;
            const double* nh = a.nHatW + 3 * wf;
            Dual sg = dual(0), sh = dual(0);
            for (int k = 0; k < D; ++k) { sg += g[k] * nh[k]; sh += h[k] * nh[k]; }
            Gbg[(long long)wf * Vp + v] = sg;
            if (a.hasH) Gbh[(long long)wf * Vp + v] = sh;
        }
    }
}

__device__ __forceinline__ Dual t_rec(const Dual* f, const Dual* G, long long c, int v, int Vp, int D, const double* d,
                                      const double* xi, double dt) {
    Dual s = f[c * Vp + v];
    Dual acc = dual(0);
    for (int k = 0; k < D; ++k) acc += G[(c * D + k) * Vp + v] * (d[k] - 0.5 * xi[k] * dt);
    return s + acc;
}

__global__ void t_recon(TArgs t, const Dual* gB, const Dual* hB, const Dual* gG, const Dual* hG, Dual* gS, Dual* hS) {
    const StepArgs& a = t.a;
    const long long n = (long long)a.nA * a.Vp;
    const int D = a.D, Vp = a.Vp;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        int f, v;
        dvi(i, Vp, f, v);
        if (v >= a.nV) continue;
        double xi[3] = {a.xi[v], a.xi[Vp + v], a.xi[2 * Vp + v]};
        const double* S = a.Sf + 3 * f;
        double xs = xi[0] * S[0] + xi[1] * S[1] + xi[2] * S[2];
        const double* dO = a.dO + 3 * f;
        if (f < a.nI) {
            const double* dN = a.dN + 3 * f;
            int o = a.own[f], nb = a.nei[f];
            if (xs >= kVSmall) {
                gS[i] = t_rec(gB, gG, o, v, Vp, D, dO, xi, a.dt);
                if (a.hasH) hS[i] = t_rec(hB, hG, o, v, Vp, D, dO, xi, a.dt);
            } else if (xs < -kVSmall) {
                gS[i] = t_rec(gB, gG, nb, v, Vp, D, dN, xi, a.dt);
                if (a.hasH) hS[i] = t_rec(hB, hG, nb, v, Vp, D, dN, xi, a.dt);
            } else {
                gS[i] = 0.5 * (t_rec(gB, gG, nb, v, Vp, D, dN, xi, a.dt) + t_rec(gB, gG, o, v, Vp, D, dO, xi, a.dt));
                if (a.hasH)
                    hS[i] = 0.5 * (t_rec(hB, hG, nb, v, Vp, D, dN, xi, a.dt) + t_rec(hB, hG, o, v, Vp, D, dO, xi, a.dt));
            }
        } else if (xs > 0) {
            int o = a.own[f];
            gS[i] = t_rec(gB, gG, o, v, Vp, D, dO, xi, a.dt);
            if (a.hasH) hS[i] = t_rec(hB, hG, o, v, Vp, D, dO, xi, a.dt);
        }
    }
}

__global__ void t_wall(TArgs t, Dual* gS, Dual* hS) {
    __shared__ double red[32 * 2];
    const StepArgs& a = t.a;
    const int wf = blockIdx.x, f = a.nI + wf, Vp = a.Vp;
    const double* S = a.Sf + 3 * f;
    double acc[2] = {0.0, 0.0};
    for (int v = threadIdx.x; v < a.nV; v += blockDim.x) {
        double xs = a.xi[v] * S[0] + a.xi[Vp + v] * S[1] + a.xi[2 * Vp + v] * S[2];
        if (xs > 0) {
            Dual r = a.w[v] * xs * gS[(long long)f * Vp + v];
            acc[0] += r.v;
            acc[1] += r.d;
        }
    }
    block_sum<2>(acc, red);
    const Dual rw = Dual{acc[0], acc[1]} / t.incAbs[wf];
    if (threadIdx.x == 0) t.rhoW[wf] = rw;
    const Dual Tw = t.Tw[wf];
    const double* Uw = a.Uw + 3 * wf;
    for (int v = threadIdx.x; v < a.nV; v += blockDim.x) {
        double x0 = a.xi[v], x1 = a.xi[Vp + v], x2 = a.xi[2 * Vp + v];
        double xs = x0 * S[0] + x1 * S[1] + x2 * S[2];
        if (xs <= 0) {
            Dual g = rw * maxwellT<Dual>(Uw[0], Uw[1], Uw[2], Tw, x0, x1, x2, a.R, a.D);
            gS[(long long)f * Vp + v] = g;
            if (a.hasH) hS[(long long)f * Vp + v] = g * (a.R * Tw) * (a.K + 3 - a.D);
        }
    }
}

template <int N>
__device__ __forceinline__ void dual_block_sum(Dual (&m)[N], double* red) {
    double x[2 * N];
    for (int i = 0; i < N; ++i) { x[2 * i] = m[i].v; x[2 * i + 1] = m[i].d; }
    block_sum<2 * N>(x, red);
    for (int i = 0; i < N; ++i) m[i] = Dual{x[2 * i], x[2 * i + 1]};
}

__global__ void t_face_mom(TArgs t, const Dual* gS, const Dual* hS) {
    __shared__ double red[32 * 30];
    const StepArgs& a = t.a;
    const int f = blockIdx.x, Vp = a.Vp;
    const long long base = (long long)f * Vp;
    Dual m[5] = {dual(0), dual(0), dual(0), dual(0), dual(0)};
    for (int v = threadIdx.x; v < a.nV; v += blockDim.x) {
        double x0 = a.xi[v], x1 = a.xi[Vp + v], x2 = a.xi[2 * Vp + v], w = a.w[v];
        Dual g = gS[base + v], h = a.hasH ? hS[base + v] : dual(0);
        m[0] += w * g;
        m[1] += w * g * x0;
        m[2] += w * g * x1;
        m[3] += w * g * x2;
        m[4] += 0.5 * w * (g * (x0 * x0 + x1 * x1 + x2 * x2) + h);
    }
    dual_block_sum<5>(m, red);
    const Dual rho = m[0];
    const Dual Ux = m[1] / rho, Uy = m[2] / rho, Uz = m[3] / rho;
    const Dual T = (m[4] - 0.5 * rho * (Ux * Ux + Uy * Uy + Uz * Uz)) / ((a.K + 3) / 2.0 * a.R * rho);
    const Dual tau = tauT<Dual>(T, rho, t.muRef, a.omega, a.Tref, a.R);
    const bool wall = f >= a.nI;
    const int wf = f - a.nI;
    Dual qq[15];
    for (int i = 0; i < 15; ++i) qq[i] = dual(0);
    double Uw0 = 0, Uw1 = 0, Uw2 = 0;
    if (wall) { Uw0 = a.Uw[3 * wf]; Uw1 = a.Uw[3 * wf + 1]; Uw2 = a.Uw[3 * wf + 2]; }
    for (int v = threadIdx.x; v < a.nV; v += blockDim.x) {
        double x0 = a.xi[v], x1 = a.xi[Vp + v], x2 = a.xi[2 * Vp + v], w = a.w[v];
        Dual g = gS[base + v], h = a.hasH ? hS[base + v] : dual(0);
        Dual c0 = x0 - Ux, c1 = x1 - Uy, c2 = x2 - Uz;
        Dual s = (c0 * c0 + c1 * c1 + c2 * c2) * g + h;
        qq[0] += 0.5 * w * c0 * s;
        qq[1] += 0.5 * w * c1 * s;
        qq[2] += 0.5 * w * c2 * s;
        if (wall) {
            double e0 = x0 - Uw0, e1 = x1 - Uw1, e2 = x2 - Uw2;
            Dual sw = (e0 * e0 + e1 * e1 + e2 * e2) * g + h;
            qq[3] += 0.5 * w * e0 * sw;
            qq[4] += 0.5 * w * e1 * sw;
            qq[5] += 0.5 * w * e2 * sw;
            Dual wg = w * g;
            qq[6] += wg * (x0 * x0); qq[7] += wg * (x0 * x1); qq[8] += wg * (x0 * x2);
            qq[9] += wg * (x1 * x0); qq[10] += wg * (x1 * x1); qq[11] += wg * (x1 * x2);
            qq[12] += wg * (x2 * x0); qq[13] += wg * (x2 * x1); qq[14] += wg * (x2 * x2);
        }
    }
    dual_block_sum<15>(qq, red);
    if (threadIdx.x == 0) {
        const double dt = a.dt;
        t.rhoF[f] = rho;
        t.UF[3 * f] = Ux; t.UF[3 * f + 1] = Uy; t.UF[3 * f + 2] = Uz;
        t.TF[f] = T;
        t.tauF[f] = tau;
        Dual fac = 2.0 * tau / (2.0 * tau + 0.5 * dt * a.Pr);
        t.qF[3 * f] = fac * qq[0]; t.qF[3 * f + 1] = fac * qq[1]; t.qF[3 * f + 2] = fac * qq[2];
        if (wall) {
            Dual fs = 2.0 * tau / (2.0 * tau + 0.5 * dt);
            for (int k = 0; k < 3; ++k) t.qWall[3 * wf + k] = fac * qq[3 + k];
            for (int k = 0; k < 9; ++k) t.stressWall[9 * wf + k] = fs * qq[6 + k];
        }
    }
}

__global__ void t_relax(TArgs t, Dual* gS, Dual* hS) {
    const StepArgs& a = t.a;
    const long long n = (long long)a.nA * a.Vp;
    const int Vp = a.Vp;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        int f, v;
        dvi(i, Vp, f, v);
        if (v >= a.nV) continue;
        double x0 = a.xi[v], x1 = a.xi[Vp + v], x2 = a.xi[2 * Vp + v];
        if (f >= a.nI) {
            const double* S = a.Sf + 3 * f;
            if (!(x0 * S[0] + x1 * S[1] + x2 * S[2] > 0)) continue;
        }
        const double hh = 0.5 * a.dt;
        Dual b = hh / (2 * t.tauF[f] + hh);
        Dual ge, he;
        shakhovT<Dual>(t.rhoF[f], t.UF[3 * f], t.UF[3 * f + 1], t.UF[3 * f + 2], t.TF[f], t.qF[3 * f], t.qF[3 * f + 1],
                       t.qF[3 * f + 2], x0, x1, x2, a.R, a.Pr, a.D, a.K, ge, he);
        gS[i] = (1.0 - b) * gS[i] + b * ge;
        if (a.hasH) hS[i] = (1.0 - b) * hS[i] + b * he;
    }
}

__global__ void t_cell(TArgs t, Dual* gT, Dual* hT, const Dual* gB, const Dual* hB, const Dual* gS, const Dual* hS) {
    const StepArgs& a = t.a;
    const long long n = (long long)a.nC * a.Vp;
    const int Vp = a.Vp;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        int c, v;
        dvi(i, Vp, c, v);
        if (v >= a.nV) continue;
        double x0 = a.xi[v], x1 = a.xi[Vp + v], x2 = a.xi[2 * Vp + v];
        const double dt = a.dt, V = a.vol[c];
        Dual g = -1.0 / 3 * gT[i] + 4.0 / 3 * gB[i];
        Dual h = a.hasH ? -1.0 / 3 * hT[i] + 4.0 / 3 * hB[i] : dual(0);
        for (int j = a.cellOff[c]; j < a.cellOff[c + 1]; ++j) {
            int e = a.cellFace[j], f = e >> 1;
            const double* S = a.Sf + 3 * f;
            double xs = x0 * S[0] + x1 * S[1] + x2 * S[2];
            long long fi = (long long)f * Vp + v;
            if (e & 1) {
                g += xs * gS[fi] * dt / V;
                if (a.hasH) h += xs * hS[fi] * dt / V;
            } else {
                g -= xs * gS[fi] * dt / V;
                if (a.hasH) h -= xs * hS[fi] * dt / V;
            }
        }
        gT[i] = g;
        if (a.hasH) hT[i] = h;
    }
}

__global__ void t_cell_mom(TArgs t, const Dual* gT, const Dual* hT) {
    __shared__ double red[32 * 10];
    const StepArgs& a = t.a;
    const int c = blockIdx.x, Vp = a.Vp;
    const long long base = (long long)c * Vp;
    Dual m[5] = {dual(0), dual(0), dual(0), dual(0), dual(0)};
    for (int v = threadIdx.x; v < a.nV; v += blockDim.x) {
        double x0 = a.xi[v], x1 = a.xi[Vp + v], x2 = a.xi[2 * Vp + v], w = a.w[v];
        Dual g = gT[base + v], h = a.hasH ? hT[base + v] : dual(0);
        m[0] += w * g;
        m[1] += w * g * x0;
        m[2] += w * g * x1;
        m[3] += w * g * x2;
        m[4] += 0.5 * w * ((x0 * x0 + x1 * x1 + x2 * x2) * g + h);
    }
    dual_block_sum<5>(m, red);
    const Dual rho = m[0];
    const Dual Ux = m[1] / rho, Uy = m[2] / rho, Uz = m[3] / rho;
    const Dual T = (m[4] - 0.5 * rho * (Ux * Ux + Uy * Uy + Uz * Uz)) / ((a.K + 3) / 2.0 * a.R * rho);
    const Dual tau = tauT<Dual>(T, rho, t.muRef, a.omega, a.Tref, a.R);
    Dual qq[3] = {dual(0), dual(0), dual(0)};
    for (int v = threadIdx.x; v < a.nV; v += blockDim.x) {
        double x0 = a.xi[v], x1 = a.xi[Vp + v], x2 = a.xi[2 * Vp + v], w = a.w[v];
        Dual g = gT[base + v], h = a.hasH ? hT[base + v] : dual(0);
        Dual c0 = x0 - Ux, c1 = x1 - Uy, c2 = x2 - Uz;
        Dual s = (c0 * c0 + c1 * c1 + c2 * c2) * g + h;
        qq[0] += 0.5 * w * c0 * s;
        qq[1] += 0.5 * w * c1 * s;
        qq[2] += 0.5 * w * c2 * s;
    }
    dual_block_sum<3>(qq, red);
    if (threadIdx.x == 0) {
        t.rho[c] = rho;
        t.U[3 * c] = Ux; t.U[3 * c + 1] = Uy; t.U[3 * c + 2] = Uz;
        t.T[c] = T;
        t.tau[c] = tau;
        Dual fac = 2.0 * tau / (2.0 * tau + a.dt * a.Pr);
        t.q[3 * c] = fac * qq[0]; t.q[3 * c + 1] = fac * qq[1]; t.q[3 * c + 2] = fac * qq[2];
        if (!(rho.v > 0.0) || !(T.v > 0.0)) atomicExch(a.status, 5);
    }
}

// J += scale * (sum_w wq_w . qWall_w + ws_w stressWall_w,xy), one block, fixed order.
template <class R>
__global__ void k_objective(int nW, const double* wq, const double* ws, const R* qWall, const R* stressWall,
                            double scale, R* J) {
    __shared__ double red[32 * 2];
    double acc[2] = {0.0, 0.0};
    for (int w = threadIdx.x; w < nW; w += blockDim.x) {
        R s = wq[3 * w] * qWall[3 * w] + wq[3 * w + 1] * qWall[3 * w + 1] + wq[3 * w + 2] * qWall[3 * w + 2] +
              ws[w] * stressWall[9 * w + 1];
        if constexpr (sizeof(R) == sizeof(double)) {
            acc[0] += (double)s;
        } else {
            acc[0] += reinterpret_cast<const Dual&>(s).v;
            acc[1] += reinterpret_cast<const Dual&>(s).d;
        }
    }
    block_sum<2>(acc, red);
    if (threadIdx.x == 0) {
        if constexpr (sizeof(R) == sizeof(double)) {
            J[0] = (double)J[0] + scale * acc[0];
        } else {
            Dual& j = reinterpret_cast<Dual&>(J[0]);
            j.v += scale * acc[0];
            j.d += scale * acc[1];
        }
    }
}

// ============================================================ adjoint
// Per-cell adjoint of the macro tuple m = (rho, Ux, Uy, Uz, T, qx, qy, qz, tau)
// (9 doubles per cell; P1 of the next step reads all nine).
constexpr int kM = 9;

struct AArgs {
    StepArgs a;
    const double* Tw;   // wall temperatures (forward values)
    double muRef;
};

// Reverse of the macro evaluation (P9 for cells, P6 for faces) for one
// entity: given lm (adjoint of rho, U, T, q, tau with q = fac(tau) Q) and the
// distributions, accumulate the adjoint of g, h and return the mu_ref part.
// facA: fac = 2 tau / (2 tau + facA) (cells: dt Pr, faces: dt Pr / 2).
// Optional wall seeds: lqw (adjoint of qWall), lsw (adjoint of stressWall) with
// fq = fac, fs = 2 tau / (2 tau + dt/2), moments about the wall velocity Uw.
__device__ void macro_reverse(const StepArgs& a, const double* g, const double* h, double* lg, double* lh,
                              const double* lm, double facA, double muRef, bool wall, const double* Uw,
                              const double* lqw, const double* lsw, double* red, double& lmu) {
    const int Vp = a.Vp;
    double m[5] = {0, 0, 0, 0, 0};
    for (int v = threadIdx.x; v < a.nV; v += blockDim.x) {
        double x0 = a.xi[v], x1 = a.xi[Vp + v], x2 = a.xi[2 * Vp + v], w = a.w[v];
        double gv = g[v], hv = a.hasH ? h[v] : 0.0;
        m[0] += w * gv;
        m[1] += w * gv * x0;
        m[2] += w * gv * x1;
        m[3] += w * gv * x2;
        m[4] += 0.5 * w * ((x0 * x0 + x1 * x1 + x2 * x2) * gv + hv);
    }
    block_sum<5>(m, red);
    __syncthreads();
    const double rho = m[0];
    const double U[3] = {m[1] / rho, m[2] / rho, m[3] / rho};
    const double cv = (a.K + 3) / 2.0 * a.R;
    const double uu = U[0] * U[0] + U[1] * U[1] + U[2] * U[2];
    const double T = (m[4] - 0.5 * rho * uu) / (cv * rho);
    const double tau = tau_ref(T, rho, muRef, a.omega, a.Tref, a.R);
    // second pass: Q_i, S0, S_ik (about U); wall: Qw_i (about Uw), stress sums
    double s2[1 + 3 + 6 + 3 + 9];
    for (int i = 0; i < 22; ++i) s2[i] = 0.0;
    for (int v = threadIdx.x; v < a.nV; v += blockDim.x) {
        double x[3] = {a.xi[v], a.xi[Vp + v], a.xi[2 * Vp + v]};
        double w = a.w[v], gv = g[v], hv = a.hasH ? h[v] : 0.0;
        double c[3] = {x[0] - U[0], x[1] - U[1], x[2] - U[2]};
        double cc = c[0] * c[0] + c[1] * c[1] + c[2] * c[2];
        double s = cc * gv + hv;
        s2[0] += w * s;
        for (int i = 0; i < 3; ++i) s2[1 + i] += 0.5 * w * c[i] * s;
        s2[4] += w * c[0] * c[0] * gv; s2[5] += w * c[0] * c[1] * gv; s2[6] += w * c[0] * c[2] * gv;
        s2[7] += w * c[1] * c[1] * gv; s2[8] += w * c[1] * c[2] * gv; s2[9] += w * c[2] * c[2] * gv;
        if (wall) {
            double e[3] = {x[0] - Uw[0], x[1] - Uw[1], x[2] - Uw[2]};
            double sw = (e[0] * e[0] + e[1] * e[1] + e[2] * e[2]) * gv + hv;
            for (int i = 0; i < 3; ++i) s2[10 + i] += 0.5 * w * e[i] * sw;
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j) s2[13 + 3 * i + j] += w * gv * x[i] * x[j];
        }
    }
    block_sum<22>(s2, red);
    const double S0 = s2[0], Q[3] = {s2[1], s2[2], s2[3]};
    const double Sik[3][3] = {{s2[4], s2[5], s2[6]}, {s2[5], s2[7], s2[8]}, {s2[6], s2[8], s2[9]}};
    // scalar chain
    const double fac = 2.0 * tau / (2.0 * tau + facA);
    const double dfac = 2.0 * facA / ((2.0 * tau + facA) * (2.0 * tau + facA));
    double lrho = lm[0], lU[3] = {lm[1], lm[2], lm[3]}, lT = lm[4], ltau = lm[8];
    double lQ[3];
    for (int i = 0; i < 3; ++i) {
        lQ[i] = lm[5 + i] * fac;
        ltau += lm[5 + i] * Q[i] * dfac;
    }
    double lQw[3] = {0, 0, 0}, lS = 0.0;
    if (wall) {
        const double fs = 2.0 * tau / (2.0 * tau + 0.5 * a.dt);
        const double dfs = 2.0 * (0.5 * a.dt) / ((2.0 * tau + 0.5 * a.dt) * (2.0 * tau + 0.5 * a.dt));
        for (int i = 0; i < 3; ++i) {
            lQw[i] = lqw[i] * fac;
            ltau += lqw[i] * s2[10 + i] * dfac;
        }
        for (int k = 0; k < 9; ++k) ltau += lsw[k] * s2[13 + k] * dfs;
        lS = fs;  // multiplies lsw in the per-DV pass
    }
    // tau = mu (T/Tref)^omega / (rho R T)
    lT += ltau * tau * (a.omega - 1.0) / T;
    lrho += -ltau * tau / rho;
    lmu += ltau * tau / muRef;
    // Q_i depends on U through c = xi - U
    for (int k = 0; k < 3; ++k)
        for (int i = 0; i < 3; ++i) lU[k] += lQ[i] * (-0.5 * ((i == k ? S0 : 0.0) + 2.0 * Sik[i][k]));
    // T = (E - rho |U|^2 / 2) / (cv rho)
    const double lE = lT / (cv * rho);
    lrho += lT * (-0.5 * uu / (cv * rho) - T / rho);
    for (int k = 0; k < 3; ++k) lU[k] += lT * (-U[k] / cv);
    // U = P / rho
    double lP[3];
    for (int k = 0; k < 3; ++k) {
        lP[k] = lU[k] / rho;
        lrho += -lU[k] * U[k] / rho;
    }
    for (int v = threadIdx.x; v < a.nV; v += blockDim.x) {
        double x[3] = {a.xi[v], a.xi[Vp + v], a.xi[2 * Vp + v]};
        double w = a.w[v];
        double c[3] = {x[0] - U[0], x[1] - U[1], x[2] - U[2]};
        double cc = c[0] * c[0] + c[1] * c[1] + c[2] * c[2];
        double xx = x[0] * x[0] + x[1] * x[1] + x[2] * x[2];
        double dg = lrho + lP[0] * x[0] + lP[1] * x[1] + lP[2] * x[2] + 0.5 * lE * xx;
        double dh = 0.5 * lE;
        for (int i = 0; i < 3; ++i) {
            dg += 0.5 * lQ[i] * c[i] * cc;
            dh += 0.5 * lQ[i] * c[i];
        }
        if (wall) {
            double e[3] = {x[0] - Uw[0], x[1] - Uw[1], x[2] - Uw[2]};
            double ee = e[0] * e[0] + e[1] * e[1] + e[2] * e[2];
            for (int i = 0; i < 3; ++i) {
                dg += 0.5 * lQw[i] * e[i] * ee;
                dh += 0.5 * lQw[i] * e[i];
            }
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j) dg += lS * lsw[3 * i + j] * x[i] * x[j];
        }
        lg[v] += w * dg;
        if (a.hasH) lh[v] += w * dh;
    }
}

// P9 reverse: one block per cell.
__global__ void r_cell_mom(AArgs A, const double* gT, const double* hT, double* lgT, double* lhT, const double* lm,
                           double* lmuC) {
    __shared__ double red[32 * 22];
    const StepArgs& a = A.a;
    const int c = blockIdx.x;
    const long long base = (long long)c * a.Vp;
    double lmu = 0.0;
    macro_reverse(a, gT + base, a.hasH ? hT + base : nullptr, lgT + base, a.hasH ? lhT + base : nullptr,
                  lm + (size_t)kM * c, a.dt * a.Pr, A.muRef, false, nullptr, nullptr, nullptr, red, lmu);
    if (threadIdx.x == 0) lmuC[c] += lmu;
}

// P8 reverse, cell part: lgT(n) = -lgT(n+1)/3, lgB = 4/3 lgT(n+1).
__global__ void r_cell_flux(AArgs A, const double* lgN, const double* lhN, double* lgT, double* lhT, double* lgB,
                            double* lhB) {
    const StepArgs& a = A.a;
    const long long n = (long long)a.nC * a.Vp;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        lgT[i] = -1.0 / 3 * lgN[i];
        lgB[i] = 4.0 / 3 * lgN[i];
        if (a.hasH) {
            lhT[i] = -1.0 / 3 * lhN[i];
            lhB[i] = 4.0 / 3 * lhN[i];
        }
    }
}

// P8 reverse, face part: adjoint of the relaxed face values.
__global__ void r_face_flux(AArgs A, const double* lgN, const double* lhN, double* lgS, double* lhS) {
    const StepArgs& a = A.a;
    const long long n = (long long)a.nA * a.Vp;
    const int Vp = a.Vp;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        int f, v;
        dvi(i, Vp, f, v);
        if (v >= a.nV) { lgS[i] = 0.0; if (a.hasH) lhS[i] = 0.0; continue; }
        const double* S = a.Sf + 3 * f;
        double xs = a.xi[v] * S[0] + a.xi[Vp + v] * S[1] + a.xi[2 * Vp + v] * S[2];
        const int o = a.own[f];
        double kg = -lgN[(long long)o * Vp + v] / a.vol[o];
        double kh = a.hasH ? -lhN[(long long)o * Vp + v] / a.vol[o] : 0.0;
        if (f < a.nI) {
            const int nb = a.nei[f];
            kg += lgN[(long long)nb * Vp + v] / a.vol[nb];
            if (a.hasH) kh += lhN[(long long)nb * Vp + v] / a.vol[nb];
        }
        lgS[i] = xs * a.dt * kg;
        if (a.hasH) lhS[i] = xs * a.dt * kh;
    }
}

// P7 + P6 reverse (+ objective seeds on walls): one block per face.  In: lgS =
// adjoint of the relaxed values; out: lgS = adjoint of the face values before
// relaxation (incoming wall DVs keep theirs for r_wall).
__global__ void r_face(AArgs A, const double* gS, const double* hS, const double* mF, double* lgS, double* lhS,
                       const double* wq, const double* ws, double objScale, double* lmuF) {
    __shared__ double red[32 * 22];
    const StepArgs& a = A.a;
    const int f = blockIdx.x, Vp = a.Vp;
    const long long base = (long long)f * Vp;
    const bool wall = f >= a.nI;
    const double* S = a.Sf + 3 * f;
    const double* m = mF + (size_t)kM * f;  // rho, U, T, q, tau of the face
    const double hh = 0.5 * a.dt;
    const double b = hh / (2.0 * m[8] + hh);
    const double db = -2.0 * hh / ((2.0 * m[8] + hh) * (2.0 * m[8] + hh));
    // P7: relaxed = (1-b) gS + b gE(mF) on relaxed DVs
    double acc[kM];
    for (int i = 0; i < kM; ++i) acc[i] = 0.0;
    ShakhovJac J;
    J.prep(m, a.R, a.Pr, a.D, a.K);
    for (int v = threadIdx.x; v < a.nV; v += blockDim.x) {
        double x0 = a.xi[v], x1 = a.xi[Vp + v], x2 = a.xi[2 * Vp + v];
        if (wall && !(x0 * S[0] + x1 * S[1] + x2 * S[2] > 0)) continue;
        double gE, hE, dg[8], dh[8];
        J.eval(x0, x1, x2, gE, hE, dg, dh);
        const double lg = lgS[base + v], lh = a.hasH ? lhS[base + v] : 0.0;
        for (int k = 0; k < 8; ++k) acc[k] += b * (dg[k] * lg + (a.hasH ? dh[k] * lh : 0.0));
        acc[8] += db * ((gE - gS[base + v]) * lg + (a.hasH ? (hE - hS[base + v]) * lh : 0.0));
        lgS[base + v] = (1.0 - b) * lg;
        if (a.hasH) lhS[base + v] = (1.0 - b) * lh;
    }
    block_sum<kM>(acc, red);
    __syncthreads();
    // P6: face macros (and wall outputs) from the face values
    double lqw[3] = {0, 0, 0}, lsw[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    const double* Uw = nullptr;
    if (wall) {
        const int wf = f - a.nI;
        Uw = a.Uw + 3 * wf;
        for (int k = 0; k < 3; ++k) lqw[k] = objScale * wq[3 * wf + k];
        lsw[1] = objScale * ws[wf];
    }
    double lmu = 0.0;
    macro_reverse(a, gS + base, a.hasH ? hS + base : nullptr, lgS + base, a.hasH ? lhS + base : nullptr, acc,
                  0.5 * a.dt * a.Pr, A.muRef, wall, Uw, lqw, lsw, red, lmu);
    if (threadIdx.x == 0) lmuF[f] += lmu;
}

// P5 + P4 reverse: one block per wall face.
__global__ void r_wall(AArgs A, const double* gS, const double* rhoW, const double* incAbs, double* lgS, double* lhS,
                       double* lTw) {
    __shared__ double red[32 * 3];
    const StepArgs& a = A.a;
    const int wf = blockIdx.x, f = a.nI + wf, Vp = a.Vp;
    const long long base = (long long)f * Vp;
    const double* S = a.Sf + 3 * f;
    const double* Uw = a.Uw + 3 * wf;
    const double Tw = A.Tw[wf], th = a.R * Tw, k3 = a.K + 3.0 - a.D;
    const double rw = rhoW[wf];
    // incoming: gS = rw M, hS = gS R Tw k3
    double acc[3] = {0.0, 0.0, 0.0};  // lrw, lTw, d incAbs / dTw
    for (int v = threadIdx.x; v < a.nV; v += blockDim.x) {
        double x0 = a.xi[v], x1 = a.xi[Vp + v], x2 = a.xi[2 * Vp + v];
        double xs = x0 * S[0] + x1 * S[1] + x2 * S[2];
        double M = maxwell_by_rho_ref(Uw[0], Uw[1], Uw[2], Tw, x0, x1, x2, a.R, a.D);
        double cc = (x0 - Uw[0]) * (x0 - Uw[0]) + (x1 - Uw[1]) * (x1 - Uw[1]) + (x2 - Uw[2]) * (x2 - Uw[2]);
        double dM = a.R * M * (cc / th - a.D) / (2.0 * th);  // dM/dTw
        if (xs <= 0) {
            const double lg = lgS[base + v], lh = a.hasH ? lhS[base + v] : 0.0;
            acc[0] += lg * M + lh * M * th * k3;
            acc[1] += rw * (lg * dM + lh * k3 * (a.R * M + th * dM));
            lgS[base + v] = 0.0;
            if (a.hasH) lhS[base + v] = 0.0;
        }
        if (xs < 0) acc[2] += -a.w[v] * xs * dM;
    }
    block_sum<3>(acc, red);
    const double lrw = acc[0];
    // rw = sum_out w xs gS / incAbs; incAbs = |sum_in -w xs M|
    const double inc = incAbs[wf];
    for (int v = threadIdx.x; v < a.nV; v += blockDim.x) {
        double xs = a.xi[v] * S[0] + a.xi[Vp + v] * S[1] + a.xi[2 * Vp + v] * S[2];
        if (xs > 0) lgS[base + v] += lrw * a.w[v] * xs / inc;
    }
    if (threadIdx.x == 0) lTw[wf] += acc[1] - lrw * rw / inc * acc[2];  // incoming sum is positive
}

// P3 reverse (+ the lagged wall gradient output G_b' = grad . n): per (cell, DV).
__global__ void r_recon(AArgs A, const double* lgS, const double* lhS, const double* lGbN, const double* lGbNh,
                        double* lgB, double* lhB, double* lG, double* lhG) {
    const StepArgs& a = A.a;
    const long long n = (long long)a.nC * a.Vp;
    const int D = a.D, Vp = a.Vp;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        int c, v;
        dvi(i, Vp, c, v);
        if (v >= a.nV) continue;
        const double xi[3] = {a.xi[v], a.xi[Vp + v], a.xi[2 * Vp + v]};
        double sb = 0.0, sbh = 0.0, gk[3] = {0, 0, 0}, hk[3] = {0, 0, 0};
        for (int j = a.cellOff[c]; j < a.cellOff[c + 1]; ++j) {
            const int e = a.cellFace[j], f = e >> 1, side = e & 1;
            const double* S = a.Sf + 3 * f;
            const double xs = xi[0] * S[0] + xi[1] * S[1] + xi[2] * S[2];
            double wgt;
            if (f < a.nI) {
                const bool up = side == 0 ? xs >= kVSmall : xs < -kVSmall;
                const bool tie = !(xs >= kVSmall) && !(xs < -kVSmall);
                wgt = up ? 1.0 : (tie ? 0.5 : 0.0);
            } else {
                wgt = xs > 0 ? 1.0 : 0.0;
            }
            if (wgt == 0.0) continue;
            const double* d = side == 0 ? a.dO + 3 * f : a.dN + 3 * f;
            const long long fi = (long long)f * Vp + v;
            const double lg = wgt * lgS[fi], lh = a.hasH ? wgt * lhS[fi] : 0.0;
            sb += lg;
            sbh += lh;
            for (int k = 0; k < D; ++k) {
                const double dk = d[k] - 0.5 * xi[k] * a.dt;
                gk[k] += lg * dk;
                hk[k] += lh * dk;
            }
        }
        // G_b' = grad . n on the wall faces of this cell
        for (int j = a.cellOff[c]; j < a.cellOff[c + 1]; ++j) {
            const int f = a.cellFace[j] >> 1;
            if (f < a.nI) continue;
            const int wf = f - a.nI;
            const double* nh = a.nHatW + 3 * wf;
            const double lb = lGbN[(long long)wf * Vp + v], lbh = a.hasH ? lGbNh[(long long)wf * Vp + v] : 0.0;
            for (int k = 0; k < D; ++k) {
                gk[k] += lb * nh[k];
                hk[k] += lbh * nh[k];
            }
        }
        lgB[i] += sb;
        if (a.hasH) lhB[i] += sbh;
        for (int k = 0; k < D; ++k) {
            lG[((long long)c * D + k) * Vp + v] = gk[k];
            if (a.hasH) lhG[((long long)c * D + k) * Vp + v] = hk[k];
        }
    }
}

// P2 reverse: lgB += transpose of the least-squares stencil; adjoint of the
// lagged wall gradient input.
__global__ void r_grad(AArgs A, const double* lG, const double* lhG, double* lgB, double* lhB, double* lGb,
                       double* lGbh) {
    const StepArgs& a = A.a;
    const long long n = (long long)a.nC * a.Vp;
    const int D = a.D, Vp = a.Vp;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        int c, v;
        dvi(i, Vp, c, v);
        if (v >= a.nV) continue;
        double sg = 0.0, sh = 0.0;
        for (int j = a.cellOff[c]; j < a.cellOff[c + 1]; ++j) {
            const int e = a.cellFace[j], f = e >> 1, side = e & 1;
            if (f < a.nI) {
                const int other = side == 0 ? a.nei[f] : a.own[f];
                const double* Lc = side == 0 ? a.pVec + 3 * f : a.nVec + 3 * f;  // this cell's vector
                const double* Lo = side == 0 ? a.nVec + 3 * f : a.pVec + 3 * f;  // the other cell's vector
                for (int k = 0; k < D; ++k) {
                    sg += Lo[k] * lG[((long long)other * D + k) * Vp + v] - Lc[k] * lG[((long long)c * D + k) * Vp + v];
                    if (a.hasH)
                        sh += Lo[k] * lhG[((long long)other * D + k) * Vp + v] - Lc[k] * lhG[((long long)c * D + k) * Vp + v];
                }
            } else {
                const int wf = f - a.nI;
                const double* L = a.bVec + 3 * wf;
                double lb = 0.0, lbh = 0.0;
                for (int k = 0; k < D; ++k) {
                    lb += L[k] * lG[((long long)c * D + k) * Vp + v];
                    if (a.hasH) lbh += L[k] * lhG[((long long)c * D + k) * Vp + v];
                }
                lGb[(long long)wf * Vp + v] = lb / a.dcW[wf];
                if (a.hasH) lGbh[(long long)wf * Vp + v] = lbh / a.dcW[wf];
            }
        }
        lgB[i] += sg;
        if (a.hasH) lhB[i] += sh;
    }
}

// P1 reverse: one block per cell.  lgT += (1-r) lgB; lm = macro adjoint of the
// cell's relaxation (rho, U, T, q, tau).
__global__ void r_barp(AArgs A, const double* gT, const double* hT, const double* mC, const double* lgB,
                       const double* lhB, double* lgT, double* lhT, double* lm) {
    __shared__ double red[32 * kM];
    const StepArgs& a = A.a;
    const int c = blockIdx.x, Vp = a.Vp;
    const long long base = (long long)c * Vp;
    const double* m = mC + (size_t)kM * c;
    const double r = 1.5 * a.dt / (2.0 * m[8] + a.dt);
    const double dr = -3.0 * a.dt / ((2.0 * m[8] + a.dt) * (2.0 * m[8] + a.dt));
    double acc[kM];
    for (int i = 0; i < kM; ++i) acc[i] = 0.0;
    ShakhovJac J;
    J.prep(m, a.R, a.Pr, a.D, a.K);
    for (int v = threadIdx.x; v < a.nV; v += blockDim.x) {
        double gE, hE, dg[8], dh[8];
        J.eval(a.xi[v], a.xi[Vp + v], a.xi[2 * Vp + v], gE, hE, dg, dh);
        const double lg = lgB[base + v], lh = a.hasH ? lhB[base + v] : 0.0;
        for (int k = 0; k < 8; ++k) acc[k] += r * (dg[k] * lg + (a.hasH ? dh[k] * lh : 0.0));
        acc[8] += dr * ((gE - gT[base + v]) * lg + (a.hasH ? (hE - hT[base + v]) * lh : 0.0));
        lgT[base + v] += (1.0 - r) * lg;
        if (a.hasH) lhT[base + v] += (1.0 - r) * lh;
    }
    block_sum<kM>(acc, red);
    if (threadIdx.x == 0)
        for (int k = 0; k < kM; ++k) lm[(size_t)kM * c + k] = acc[k];
}

// Pack cell / face macros of the forward pass as (rho, U, T, q, tau) tuples.
__global__ void k_pack_macros(int n, const double* rho, const double* U, const double* T, const double* q,
                              const double* tau, double* out) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double* o = out + (size_t)kM * i;
        o[0] = rho[i];
        for (int k = 0; k < 3; ++k) { o[1 + k] = U[3 * i + k]; o[5 + k] = q[3 * i + k]; }
        o[4] = T[i];
        o[8] = tau[i];
    }
}

__global__ void k_sum(int n, const double* x, double* out) {  // one block, fixed order
    __shared__ double red[32];
    double s[1] = {0.0};
    for (int i = threadIdx.x; i < n; i += blockDim.x) s[0] += x[i];
    block_sum<1>(s, red);
    if (threadIdx.x == 0) out[0] += s[0];
}

}  // namespace

// ------------------------------------------------------------ launchers
void tlm_launch_incabs(const TlmState& s, cudaStream_t st) {
    TArgs t{s.a, s.rho, s.U, s.T, s.q, s.tau, s.rhoF, s.UF, s.TF, s.qF, s.tauF, s.rhoW, s.qWall, s.stressWall,
            s.Tw, s.incAbs, s.muRef};
    t_incabs<<<s.a.nW, kRT, 0, st>>>(t);
}
void tlm_launch_init(const TlmState& s, const double* rho0, const double* U0, const double* T0, int sms,
                     cudaStream_t st) {
    TArgs t{s.a, s.rho, s.U, s.T, s.q, s.tau, s.rhoF, s.UF, s.TF, s.qF, s.tauF, s.rhoW, s.qWall, s.stressWall,
            s.Tw, s.incAbs, s.muRef};
    t_init<<<grid((long long)s.a.nC * s.a.Vp, kT, sms), kT, 0, st>>>(t, rho0, U0, T0, s.gT, s.hT);
    cudaMemsetAsync(s.Gbg, 0, sizeof(Dual) * (size_t)s.a.nW * s.a.Vp, st);
    if (s.a.hasH) cudaMemsetAsync(s.Gbh, 0, sizeof(Dual) * (size_t)s.a.nW * s.a.Vp, st);
}
void tlm_launch_step(const TlmState& s, bool objective, const double* wq, const double* ws, double scale, Dual* J,
                     int sms, cudaStream_t st) {
    TArgs t{s.a, s.rho, s.U, s.T, s.q, s.tau, s.rhoF, s.UF, s.TF, s.qF, s.tauF, s.rhoW, s.qWall, s.stressWall,
            s.Tw, s.incAbs, s.muRef};
    const StepArgs& a = s.a;
    const long long nCV = (long long)a.nC * a.Vp, nAV = (long long)a.nA * a.Vp;
    t_barp<<<grid(nCV, kT, sms), kT, 0, st>>>(t, s.gT, s.hT, s.gB, s.hB);
    t_grad<<<grid(nCV, kT, sms), kT, 0, st>>>(t, s.gB, s.hB, s.gG, s.hG, s.Gbg, s.Gbh);
    t_recon<<<grid(nAV, kT, sms), kT, 0, st>>>(t, s.gB, s.hB, s.gG, s.hG, s.gS, s.hS);
    if (a.nW > 0) t_wall<<<a.nW, kRT, 0, st>>>(t, s.gS, s.hS);
    t_face_mom<<<a.nA, kRT, 0, st>>>(t, s.gS, s.hS);
    if (objective && a.nW > 0) k_objective<Dual><<<1, kT, 0, st>>>(a.nW, wq, ws, s.qWall, s.stressWall, scale, J);
    t_relax<<<grid(nAV, kT, sms), kT, 0, st>>>(t, s.gS, s.hS);
    t_cell<<<grid(nCV, kT, sms), kT, 0, st>>>(t, s.gT, s.hT, s.gB, s.hB, s.gS, s.hS);
    t_cell_mom<<<a.nC, kRT, 0, st>>>(t, s.gT, s.hT);
}

void launch_objective(const StepArgs& a, const double* wq, const double* ws, double scale, double* J, cudaStream_t st) {
    if (a.nW > 0) k_objective<double><<<1, kT, 0, st>>>(a.nW, wq, ws, a.qWall, a.stressWall, scale, J);
}

void adj_pack_macros(int n, const double* rho, const double* U, const double* T, const double* q, const double* tau,
                     double* out, int sms, cudaStream_t st) {
    k_pack_macros<<<grid(n, kT, sms), kT, 0, st>>>(n, rho, U, T, q, tau, out);
}

void adj_launch_step(const AdjState& s, const double* gTn, const double* hTn, bool objective, const double* wq,
                     const double* ws, double scale, int sms, cudaStream_t st) {
    AArgs A{s.a, s.a.Tw, s.muRef};
    const StepArgs& a = s.a;
    const long long nCV = (long long)a.nC * a.Vp, nAV = (long long)a.nA * a.Vp;
    // P9 reverse: lgN += J9^T lmN (state n+1 and the adjoint of its macros)
    if (s.haveMacroAdj) r_cell_mom<<<a.nC, kRT, 0, st>>>(A, gTn, hTn, s.lgN, s.lhN, s.lmN, s.lmuC);
    // P8 reverse
    r_cell_flux<<<grid(nCV, kT, sms), kT, 0, st>>>(A, s.lgN, s.lhN, s.lgT, s.lhT, s.lgB, s.lhB);
    r_face_flux<<<grid(nAV, kT, sms), kT, 0, st>>>(A, s.lgN, s.lhN, s.lgS, s.lhS);
    // P7 + P6 reverse
    r_face<<<a.nA, kRT, 0, st>>>(A, s.gS, s.hS, s.mF, s.lgS, s.lhS, s.wq, s.ws, objective ? scale : 0.0, s.lmuF);
    // P5 + P4 reverse
    if (a.nW > 0) r_wall<<<a.nW, kRT, 0, st>>>(A, s.gS, a.rhoW, a.incAbs, s.lgS, s.lhS, s.lTw);
    // P3 reverse (+ G_b' = grad.n), P2 reverse
    r_recon<<<grid(nCV, kT, sms), kT, 0, st>>>(A, s.lgS, s.lhS, s.lGbN, s.lGbNh, s.lgB, s.lhB, s.lG, s.lhG);
    r_grad<<<grid(nCV, kT, sms), kT, 0, st>>>(A, s.lG, s.lhG, s.lgB, s.lhB, s.lGb, s.lGbh);
    // P1 reverse
    r_barp<<<a.nC, kRT, 0, st>>>(A, s.gT, s.hT, s.mC, s.lgB, s.lhB, s.lgT, s.lhT, s.lm);
    (void)wq;
    (void)ws;
}

void adj_sum(int n, const double* x, double* out, cudaStream_t st) { k_sum<<<1, kT, 0, st>>>(n, x, out); }

}  // namespace dugks
