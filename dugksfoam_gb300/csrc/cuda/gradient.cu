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
constexpr int kAW = 4;  // warps per block of the warp-per-entity reverse kernels

struct AArgs {
    StepArgs a;
    const double* Tw;   // wall temperatures (forward values)
    double muRef;
    int M;              // velocities per direction: v = (iz M + iy) M + ix (fvDVM.C:151-221)
};

// Butterfly sum of N values over the warp; every lane gets the totals (fixed
// order, so the result does not depend on the launch).
template <int N>
__device__ __forceinline__ void wsum(double* v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
#pragma unroll
        for (int i = 0; i < N; ++i) v[i] += __shfl_xor_sync(0xffffffffu, v[i], o);
}

// Tensor-product position (ix, iy, iz) of velocity v, advanced by a lane stride.
template <int D>
struct DvIdx {
    int ix, iy, iz;
    __device__ __forceinline__ void init(int v, int M) {
        ix = v % M;
        const int r = v / M;
        iy = D == 3 ? r % M : r;
        iz = D == 3 ? r / M : 0;
    }
    __device__ __forceinline__ void advance(int s, int M) {
        ix += s;
        while (ix >= M) { ix -= M; ++iy; }
        if (D == 3)
            while (iy >= M) { iy -= M; ++iz; }
    }
};

// exp(-(xi_d - U_d)^2 / (2 theta)) for the M abscissae of every direction of
// the tensor-product grid, so that the Maxwellian factor of velocity
// (ix, iy, iz) is N E[ix] E[M + iy] E[2M + iz]: D M exponentials per entity
// instead of one per velocity.  E holds D*M doubles of this warp.
template <int D>
__device__ __forceinline__ void gauss_table(const StepArgs& a, int M, const double* U, double ith, double* E) {
    const int lane = threadIdx.x & 31;
    __syncwarp();  // the previous entity's reads of E are done
    for (int i = lane; i < M; i += 32) {
        const double c0 = a.xi[i] - U[0];                    // x of velocity (i, 0, 0)
        E[i] = exp(-0.5 * (c0 * c0 * ith));
        const double c1 = a.xi[a.Vp + i * M] - U[1];        // y of velocity (0, i, 0)
        E[M + i] = exp(-0.5 * (c1 * c1 * ith));
        if (D == 3) {
            const double c2 = a.xi[2 * a.Vp + i * M * M] - U[2];  // z of velocity (0, 0, i)
            E[2 * M + i] = exp(-0.5 * (c2 * c2 * ith));
        }
    }
    __syncwarp();
}

// Transposed Jacobian of the Shakhov equilibrium (gE, hE)(rho, U, T, q)
// applied to one velocity's adjoints (lg, lh).  With theta = R T, c = xi - U,
// a = |c|^2/theta, G0 = (2 pi theta)^(-D/2) exp(-a/2), kap = (1-Pr)/(5 theta^2),
// k3 = K+3-D, B = (a-D) k3 - 2K, P = a-D-2:
//   gE = rho G0 + kap (c.q) P G0,   hE = theta [k3 rho G0 + kap (c.q) B G0]
//   dgE/drho = G0,                          dhE/drho = theta k3 G0
//   dgE/dU_k = gU c_k/theta - kap G0 q_k P,  gU = rho G0 + kap (c.q)(P-2) G0
//   dhE/dU_k = hU c_k - theta kap G0 q_k B,  hU = k3 rho G0 + kap (c.q)(B-2 k3) G0
//   dgE/dq_k = kap G0 c_k P,                dhE/dq_k = theta kap G0 c_k B
//   dG0/dtheta = G0 (a-D) / (2 theta).
// Accumulators (NJ = 2D+4): J[0] rho; J[1..D] sum c_k t1; J[D+1] sum t2 (the
// U_k part -q_k t2 is applied once in finish); J[D+2..2D+1] q; J[2D+2] theta;
// J[2D+3] sum (gE-g) lg + (hE-h) lh (the relaxation-rate part).
template <int D>
struct ShakhovJacT {
    static constexpr int NJ = 2 * D + 4;
    double rho, U[3], q[3], th, ith, N, kap, k3, K2;
    __device__ __forceinline__ void prep(const double* m, double Rg, double Pr, int K) {
        rho = m[0];
        for (int k = 0; k < 3; ++k) { U[k] = m[1 + k]; q[k] = m[5 + k]; }
        th = Rg * m[4];
        ith = 1.0 / th;
        const double s = sqrt(2.0 * kPi * th);
        N = 1.0 / (D == 2 ? s * s : s * s * s);
        kap = (1.0 - Pr) / 5.0 * ith * ith;
        k3 = K + 3.0 - D;
        K2 = 2.0 * K;
    }
    __device__ __forceinline__ void apply(const double* c, double cc, double G0, double g, double h, double lg,
                                          double lh, double* J) const {
        double cq = 0.0;
#pragma unroll
        for (int k = 0; k < D; ++k) cq += c[k] * q[k];
        const double a = cc * ith;
        const double P = a - D - 2.0, B = (a - D) * k3 - K2;
        const double rG = rho * G0, kG = kap * G0, kGcq = kG * cq;
        const double gE = rG + kGcq * P;
        const double H = k3 * rG + kGcq * B;
        const double hE = th * H;
        const double gU = rG + kGcq * (P - 2.0), hU = k3 * rG + kGcq * (B - 2.0 * k3);
        const double t1 = gU * ith * lg + hU * lh;
        const double t2 = kG * (P * lg + th * B * lh);
        J[0] += G0 * (lg + th * k3 * lh);
#pragma unroll
        for (int k = 0; k < D; ++k) J[1 + k] += c[k] * t1;
        J[D + 1] += t2;
#pragma unroll
        for (int k = 0; k < D; ++k) J[D + 2 + k] += c[k] * t2;
        const double hd = 0.5 * (a - D) * ith;
        const double dgth = rG * hd + kGcq * ith * (-2.0 * P - a + P * (a - D) * 0.5);
        const double dHth = k3 * rG * hd + kGcq * ith * (-2.0 * B - k3 * a + B * (a - D) * 0.5);
        J[2 * D + 2] += dgth * lg + (H + th * dHth) * lh;
        J[2 * D + 3] += (gE - g) * lg + (hE - h) * lh;
    }
    // Adjoint of (rho, U, T, q, tau) from the summed accumulators; s scales the
    // equilibrium part (the relaxation weight), ds the rate part (d weight/d tau).
    __device__ __forceinline__ void finish(const double* J, double s, double ds, double Rg, double* lm) const {
        lm[0] = s * J[0];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            lm[1 + k] = k < D ? s * (J[1 + k] - q[k] * J[D + 1]) : 0.0;
            lm[5 + k] = k < D ? s * J[D + 2 + k] : 0.0;
        }
        lm[4] = s * (Rg * J[2 * D + 2]);
        lm[8] = ds * J[2 * D + 3];
    }
};

// Second moments of one entity about its velocity U (and, on walls, about the
// wall velocity Uw) that the macro reverse needs:
//   S0 = sum w (|c|^2 g + h),  Q_i = 1/2 sum w c_i (|c|^2 g + h),  S_ij = sum w c_i c_j g (i <= j)
//   wall: Qw_i = 1/2 sum w e_i (|e|^2 g + h) (e = xi - Uw),  X_ij = sum w xi_i xi_j g.
template <int D>
struct Mom2 {
    static constexpr int NS = D * (D + 1) / 2;
    static constexpr int N = 1 + D + NS;
    static constexpr int NWALL = D + D * D;
    static __device__ __forceinline__ constexpr int sidx(int i, int j) {  // upper triangle, row-major
        return i <= j ? i * D - i * (i - 1) / 2 + (j - i) : j * D - j * (j - 1) / 2 + (i - j);
    }
    static __device__ __forceinline__ void add(const double* c, double cc, double w, double g, double h, double* s) {
        const double ws = w * (cc * g + h), wg = w * g;
        s[0] += ws;
#pragma unroll
        for (int i = 0; i < D; ++i) s[1 + i] += 0.5 * ws * c[i];
#pragma unroll
        for (int i = 0; i < D; ++i)
#pragma unroll
            for (int j = i; j < D; ++j) s[1 + D + sidx(i, j)] += wg * c[i] * c[j];
    }
    static __device__ __forceinline__ void add_wall(const double* x, const double* Uw, double w, double g, double h,
                                                    double* s) {
        double e[D], ee = 0.0;
#pragma unroll
        for (int i = 0; i < D; ++i) { e[i] = x[i] - Uw[i]; ee += e[i] * e[i]; }
        const double sw = w * (ee * g + h), wg = w * g;
#pragma unroll
        for (int i = 0; i < D; ++i) s[i] += 0.5 * sw * e[i];
#pragma unroll
        for (int i = 0; i < D; ++i)
#pragma unroll
            for (int j = 0; j < D; ++j) s[D + D * i + j] += wg * x[i] * x[j];
    }
};

// Reverse of the macro evaluation of one entity (P9 for cells, P6 for faces;
// fvDVM::updateMacroVol fvDVM.C:597-728, updateMacroSurf :456-582).  Inputs:
// the forward macros (rho, U, T, tau) of the entity, lm = adjoint of
// (rho, U, T, q, tau) with q = fac(tau) Q and fac = 2 tau / (2 tau + facA)
// (cells facA = dt Pr, faces dt Pr / 2), the second moments s (Mom2 layout,
// wall part after the first Mom2::N), and on walls the seeds lqw (adjoint of
// qWall = fac Qw) and lsw (adjoint of stressWall = fs X, fs = 2 tau / (2 tau + dt/2)).
// Output: per-velocity coefficients so that
//   lg += w [lrho + lP.xi + lE/2 |xi|^2 + 1/2 (lQ.c)|c|^2 + 1/2 (lQw.e)|e|^2 + xi.lX.xi]
//   lh += w [lE/2 + 1/2 lQ.c + 1/2 lQw.e],
// and the mu_ref adjoint (tau = mu_ref (T/Tref)^omega / (rho R T)).
template <int D>
struct MacroAdj {
    double lrho, lP[D], hE, hQ[D], hQw[D], lX[D * D], U[D], Uw[D];
    bool wall;
    __device__ __forceinline__ double chain(const StepArgs& a, double rho, const double* Um, double T, double tau,
                                            const double* lm, const double* s, double facA, double muRef, bool isWall,
                                            const double* Uwall, const double* lqw, const double* lsw) {
        using M2 = Mom2<D>;
        wall = isWall;
        const double cv = (a.K + 3) / 2.0 * a.R;
        double uu = 0.0;
#pragma unroll
        for (int k = 0; k < D; ++k) { U[k] = Um[k]; uu += U[k] * U[k]; }
        const double fac = 2.0 * tau / (2.0 * tau + facA);
        const double dfac = 2.0 * facA / ((2.0 * tau + facA) * (2.0 * tau + facA));
        double lU[D], lQ[D], lT = lm[4], ltau = lm[8];
        lrho = lm[0];
#pragma unroll
        for (int i = 0; i < D; ++i) {
            lU[i] = lm[1 + i];
            lQ[i] = lm[5 + i] * fac;
            ltau += lm[5 + i] * s[1 + i] * dfac;
        }
        if (wall) {
            const double fs = 2.0 * tau / (2.0 * tau + 0.5 * a.dt);
            const double dfs = 2.0 * (0.5 * a.dt) / ((2.0 * tau + 0.5 * a.dt) * (2.0 * tau + 0.5 * a.dt));
            const double* sw = s + M2::N;
#pragma unroll
            for (int i = 0; i < D; ++i) {
                Uw[i] = Uwall[i];
                hQw[i] = 0.5 * (lqw[i] * fac);
                ltau += lqw[i] * sw[i] * dfac;
            }
#pragma unroll
            for (int i = 0; i < D; ++i)
#pragma unroll
                for (int j = 0; j < D; ++j) {
                    ltau += lsw[3 * i + j] * sw[D + D * i + j] * dfs;
                    lX[D * i + j] = fs * lsw[3 * i + j];
                }
        }
        lT += ltau * tau * (a.omega - 1.0) / T;
        lrho += -ltau * tau / rho;
        const double lmu = ltau * tau / muRef;
        // Q_i depends on U through c = xi - U
        const double S0 = s[0];
#pragma unroll
        for (int k = 0; k < D; ++k)
#pragma unroll
            for (int i = 0; i < D; ++i)
                lU[k] += lQ[i] * (-0.5 * ((i == k ? S0 : 0.0) + 2.0 * s[1 + D + M2::sidx(i, k)]));
        // T = (E - rho |U|^2 / 2) / (cv rho)
        const double lE = lT / (cv * rho);
        lrho += lT * (-0.5 * uu / (cv * rho) - T / rho);
#pragma unroll
        for (int k = 0; k < D; ++k) lU[k] += lT * (-U[k] / cv);
        // U = P / rho
#pragma unroll
        for (int k = 0; k < D; ++k) {
            lP[k] = lU[k] / rho;
            lrho += -lU[k] * U[k] / rho;
        }
        hE = 0.5 * lE;
#pragma unroll
        for (int i = 0; i < D; ++i) hQ[i] = 0.5 * lQ[i];
        return lmu;
    }
    __device__ __forceinline__ void dgh(const double* x, double& dg, double& dh) const {
        double c[D], cc = 0.0, xx = 0.0, lc = 0.0;
        dg = lrho;
#pragma unroll
        for (int k = 0; k < D; ++k) {
            c[k] = x[k] - U[k];
            cc += c[k] * c[k];
            xx += x[k] * x[k];
            dg += lP[k] * x[k];
            lc += hQ[k] * c[k];
        }
        dg += hE * xx + lc * cc;
        dh = hE + lc;
        if (wall) {
            double e[D], ee = 0.0, le = 0.0;
#pragma unroll
            for (int k = 0; k < D; ++k) {
                e[k] = x[k] - Uw[k];
                ee += e[k] * e[k];
                le += hQw[k] * e[k];
            }
            dg += le * ee;
            dh += le;
#pragma unroll
            for (int i = 0; i < D; ++i)
#pragma unroll
                for (int j = 0; j < D; ++j) dg += lX[D * i + j] * x[i] * x[j];
        }
    }
};

template <int D>
__device__ __forceinline__ void load_xi(const StepArgs& a, int v, double* x) {
#pragma unroll
    for (int k = 0; k < D; ++k) x[k] = a.xi[k * a.Vp + v];
}

// P9 reverse fused with the cell part of P8: one warp per cell.  lgN (adjoint
// of state n+1) += J9^T lmN; then lgT(n) = -lgN/3 and lgB = 4/3 lgN.  mN holds
// the macros of state n+1 as stored (rho [nC], U [nC][3], T [nC], q [nC][3], tau [nC]).
template <int D, bool HH>
__global__ void __launch_bounds__(kAW * 32) r_cell_mom(AArgs A, const double* gT, const double* hT, const double* mN,
                                                       double* lgN, double* lhN, double* lgT, double* lhT,
                                                       double* lgB, double* lhB, const double* lmN, double* lmuC) {
    using M2 = Mom2<D>;
    const StepArgs& a = A.a;
    const int lane = threadIdx.x & 31, Vp = a.Vp, nC = a.nC;
    for (int c = blockIdx.x * kAW + (threadIdx.x >> 5); c < nC; c += gridDim.x * kAW) {
        const long long base = (long long)c * Vp;
        const double rho = mN[c], T = mN[4 * nC + c], tau = mN[8 * nC + c];
        double U[D];
#pragma unroll
        for (int k = 0; k < D; ++k) U[k] = mN[nC + 3 * c + k];
        double s[M2::N];
#pragma unroll
        for (int i = 0; i < M2::N; ++i) s[i] = 0.0;
        for (int v = lane; v < a.nV; v += 32) {
            double x[D], cv[D], cc = 0.0;
            load_xi<D>(a, v, x);
#pragma unroll
            for (int k = 0; k < D; ++k) { cv[k] = x[k] - U[k]; cc += cv[k] * cv[k]; }
            M2::add(cv, cc, a.w[v], gT[base + v], HH ? hT[base + v] : 0.0, s);
        }
        wsum<M2::N>(s);
        MacroAdj<D> o;
        const double lmu = o.chain(a, rho, U, T, tau, lmN + (size_t)kM * c, s, a.dt * a.Pr, A.muRef, false, nullptr,
                                   nullptr, nullptr);
        for (int v = lane; v < Vp; v += 32) {  // padding: w = 0, the copies below still run
            double x[D], dg, dh;
            load_xi<D>(a, v, x);
            o.dgh(x, dg, dh);
            const double w = a.w[v];
            const double lg = lgN[base + v] + w * dg;
            lgN[base + v] = lg;
            lgT[base + v] = -1.0 / 3 * lg;
            lgB[base + v] = 4.0 / 3 * lg;
            if (HH) {
                const double lh = lhN[base + v] + w * dh;
                lhN[base + v] = lh;
                lhT[base + v] = -1.0 / 3 * lh;
                lhB[base + v] = 4.0 / 3 * lh;
            }
        }
        if (lane == 0) lmuC[c] += lmu;
    }
}

// P8 reverse, cell part alone (the last step, where the macros of n+1 carry no
// adjoint): lgT(n) = -lgT(n+1)/3, lgB = 4/3 lgT(n+1).
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

// P8 reverse, face part: adjoint of the relaxed face values; one warp per face.
template <int D, bool HH>
__global__ void __launch_bounds__(kAW * 32) r_face_flux(AArgs A, const double* lgN, const double* lhN, double* lgS,
                                                        double* lhS) {
    const StepArgs& a = A.a;
    const int lane = threadIdx.x & 31, Vp = a.Vp;
    for (int f = blockIdx.x * kAW + (threadIdx.x >> 5); f < a.nA; f += gridDim.x * kAW) {
        const long long base = (long long)f * Vp;
        const double* S = a.Sf + 3 * f;
        const int o = a.own[f];
        const bool inner = f < a.nI;
        const int nb = inner ? a.nei[f] : o;
        const double iVo = 1.0 / a.vol[o], iVn = inner ? 1.0 / a.vol[nb] : 0.0;
        const double* lgo = lgN + (long long)o * Vp;
        const double* lgn = lgN + (long long)nb * Vp;
        for (int v = lane; v < Vp; v += 32) {
            if (v >= a.nV) {
                lgS[base + v] = 0.0;
                if (HH) lhS[base + v] = 0.0;
                continue;
            }
            double x[D], xs = 0.0;
            load_xi<D>(a, v, x);
#pragma unroll
            for (int k = 0; k < D; ++k) xs += x[k] * S[k];
            double kg = -lgo[v] * iVo;
            if (inner) kg += lgn[v] * iVn;
            lgS[base + v] = xs * a.dt * kg;
            if (HH) {
                double kh = -lhN[(long long)o * Vp + v] * iVo;
                if (inner) kh += lhN[(long long)nb * Vp + v] * iVn;
                lhS[base + v] = xs * a.dt * kh;
            }
        }
    }
}

// P7 + P6 reverse (+ objective seeds on walls): one warp per face.  In: lgS =
// adjoint of the relaxed values; out: lgS = adjoint of the face values before
// relaxation (incoming wall DVs keep theirs for r_wall).  mF: forward face
// macros (rho, U, T, q, tau) of the step.  One pass over the velocities forms
// the Shakhov Jacobian product and the second moments together; a second pass
// writes the adjoints.
template <int D, bool HH>
__global__ void __launch_bounds__(kAW * 32) r_face(AArgs A, const double* gS, const double* hS, const double* mF,
                                                   double* lgS, double* lhS, const double* wq, const double* ws,
                                                   double objScale, double* lmuF) {
    using SJ = ShakhovJacT<D>;
    using M2 = Mom2<D>;
    constexpr int NA = SJ::NJ + M2::N, NT = NA + M2::NWALL;
    extern __shared__ double eTab[];
    const StepArgs& a = A.a;
    const int lane = threadIdx.x & 31, Vp = a.Vp, M = A.M;
    double* E = eTab + (threadIdx.x >> 5) * D * M;
    const double hh = 0.5 * a.dt;
    for (int f = blockIdx.x * kAW + (threadIdx.x >> 5); f < a.nA; f += gridDim.x * kAW) {
        const long long base = (long long)f * Vp;
        const bool wall = f >= a.nI;
        const double* S = a.Sf + 3 * f;
        const double* m = mF + (size_t)kM * f;
        const double* Uw = wall ? a.Uw + 3 * (f - a.nI) : nullptr;
        SJ J;
        J.prep(m, a.R, a.Pr, a.K);
        const double b = hh / (2.0 * m[8] + hh);
        const double db = -2.0 * hh / ((2.0 * m[8] + hh) * (2.0 * m[8] + hh));
        gauss_table<D>(a, M, J.U, J.ith, E);
        double acc[NT];
#pragma unroll
        for (int i = 0; i < NT; ++i) acc[i] = 0.0;
        DvIdx<D> id;
        id.init(lane, M);
        for (int v = lane; v < a.nV; v += 32, id.advance(32, M)) {
            double x[D], c[D], cc = 0.0, xs = 0.0;
            load_xi<D>(a, v, x);
#pragma unroll
            for (int k = 0; k < D; ++k) {
                c[k] = x[k] - J.U[k];
                cc += c[k] * c[k];
                xs += x[k] * S[k];
            }
            const double g = gS[base + v], h = HH ? hS[base + v] : 0.0;
            if (!wall || xs > 0) {  // relaxed velocities (walls: outgoing only)
                double G0 = J.N * E[id.ix] * E[M + id.iy];
                if (D == 3) G0 *= E[2 * M + id.iz];
                J.apply(c, cc, G0, g, h, lgS[base + v], HH ? lhS[base + v] : 0.0, acc);
            }
            M2::add(c, cc, a.w[v], g, h, acc + SJ::NJ);
            if (wall) M2::add_wall(x, Uw, a.w[v], g, h, acc + NA);
        }
        if (wall) wsum<NT>(acc);
        else wsum<NA>(acc);
        double lm[kM];
        J.finish(acc, b, db, a.R, lm);
        double lqw[3] = {0.0, 0.0, 0.0}, lsw[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
        if (wall) {
            const int wf = f - a.nI;
            for (int k = 0; k < 3; ++k) lqw[k] = objScale * wq[3 * wf + k];
            lsw[1] = objScale * ws[wf];
        }
        MacroAdj<D> o;
        const double lmu = o.chain(a, m[0], J.U, m[4], m[8], lm, acc + SJ::NJ, 0.5 * a.dt * a.Pr, A.muRef, wall, Uw,
                                   lqw, lsw);
        for (int v = lane; v < a.nV; v += 32) {
            double x[D], dg, dh, xs = 0.0;
            load_xi<D>(a, v, x);
#pragma unroll
            for (int k = 0; k < D; ++k) xs += x[k] * S[k];
            o.dgh(x, dg, dh);
            const double w = a.w[v];
            const bool relaxed = !wall || xs > 0;
            double lg = lgS[base + v];
            if (relaxed) lg = (1.0 - b) * lg;
            lgS[base + v] = lg + w * dg;
            if (HH) {
                double lh = lhS[base + v];
                if (relaxed) lh = (1.0 - b) * lh;
                lhS[base + v] = lh + w * dh;
            }
        }
        if (lane == 0) lmuF[f] += lmu;
    }
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

// P3 reverse (+ the lagged wall gradient output G_b' = grad . n): one warp per cell.
template <int D, bool HH>
__global__ void __launch_bounds__(kAW * 32) r_recon(AArgs A, const double* lgS, const double* lhS,
                                                    const double* lGbN, const double* lGbNh, double* lgB, double* lhB,
                                                    double* lG, double* lhG) {
    const StepArgs& a = A.a;
    const int lane = threadIdx.x & 31, Vp = a.Vp;
    for (int c = blockIdx.x * kAW + (threadIdx.x >> 5); c < a.nC; c += gridDim.x * kAW) {
        const int j0 = a.cellOff[c], j1 = a.cellOff[c + 1];
        const long long base = (long long)c * Vp;
        for (int v = lane; v < a.nV; v += 32) {
            double xi[D];
            load_xi<D>(a, v, xi);
            double sb = 0.0, sbh = 0.0, gk[D], hk[D];
#pragma unroll
            for (int k = 0; k < D; ++k) gk[k] = hk[k] = 0.0;
            for (int j = j0; j < j1; ++j) {
                const int e = a.cellFace[j], f = e >> 1, side = e & 1;
                const double* S = a.Sf + 3 * f;
                double xs = 0.0;
#pragma unroll
                for (int k = 0; k < D; ++k) xs += xi[k] * S[k];
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
                const double lg = wgt * lgS[fi], lh = HH ? wgt * lhS[fi] : 0.0;
                sb += lg;
                sbh += lh;
#pragma unroll
                for (int k = 0; k < D; ++k) {
                    const double dk = d[k] - 0.5 * xi[k] * a.dt;
                    gk[k] += lg * dk;
                    hk[k] += lh * dk;
                }
            }
            // G_b' = grad . n on the wall faces of this cell
            for (int j = j0; j < j1; ++j) {
                const int f = a.cellFace[j] >> 1;
                if (f < a.nI) continue;
                const int wf = f - a.nI;
                const double* nh = a.nHatW + 3 * wf;
                const double lb = lGbN[(long long)wf * Vp + v], lbh = HH ? lGbNh[(long long)wf * Vp + v] : 0.0;
#pragma unroll
                for (int k = 0; k < D; ++k) {
                    gk[k] += lb * nh[k];
                    hk[k] += lbh * nh[k];
                }
            }
            lgB[base + v] += sb;
            if (HH) lhB[base + v] += sbh;
#pragma unroll
            for (int k = 0; k < D; ++k) {
                lG[((long long)c * D + k) * Vp + v] = gk[k];
                if (HH) lhG[((long long)c * D + k) * Vp + v] = hk[k];
            }
        }
    }
}

// P2 reverse: lgB += transpose of the least-squares stencil; adjoint of the
// lagged wall gradient input.  One warp per cell.
template <int D, bool HH>
__global__ void __launch_bounds__(kAW * 32) r_grad(AArgs A, const double* lG, const double* lhG, double* lgB,
                                                   double* lhB, double* lGb, double* lGbh) {
    const StepArgs& a = A.a;
    const int lane = threadIdx.x & 31, Vp = a.Vp;
    for (int c = blockIdx.x * kAW + (threadIdx.x >> 5); c < a.nC; c += gridDim.x * kAW) {
        const int j0 = a.cellOff[c], j1 = a.cellOff[c + 1];
        const long long base = (long long)c * Vp;
        for (int v = lane; v < a.nV; v += 32) {
            double sg = 0.0, sh = 0.0;
            for (int j = j0; j < j1; ++j) {
                const int e = a.cellFace[j], f = e >> 1, side = e & 1;
                if (f < a.nI) {
                    const int other = side == 0 ? a.nei[f] : a.own[f];
                    const double* Lc = side == 0 ? a.pVec + 3 * f : a.nVec + 3 * f;  // this cell's vector
                    const double* Lo = side == 0 ? a.nVec + 3 * f : a.pVec + 3 * f;  // the other cell's vector
#pragma unroll
                    for (int k = 0; k < D; ++k) {
                        sg += Lo[k] * lG[((long long)other * D + k) * Vp + v] - Lc[k] * lG[((long long)c * D + k) * Vp + v];
                        if (HH)
                            sh += Lo[k] * lhG[((long long)other * D + k) * Vp + v] -
                                  Lc[k] * lhG[((long long)c * D + k) * Vp + v];
                    }
                } else {
                    const int wf = f - a.nI;
                    const double* L = a.bVec + 3 * wf;
                    double lb = 0.0, lbh = 0.0;
#pragma unroll
                    for (int k = 0; k < D; ++k) {
                        lb += L[k] * lG[((long long)c * D + k) * Vp + v];
                        if (HH) lbh += L[k] * lhG[((long long)c * D + k) * Vp + v];
                    }
                    lGb[(long long)wf * Vp + v] = lb / a.dcW[wf];
                    if (HH) lGbh[(long long)wf * Vp + v] = lbh / a.dcW[wf];
                }
            }
            lgB[base + v] += sg;
            if (HH) lhB[base + v] += sh;
        }
    }
}

// P1 reverse: one warp per cell.  lgT += (1-r) lgB; lm = macro adjoint of the
// cell's relaxation (rho, U, T, q, tau).
template <int D, bool HH>
__global__ void __launch_bounds__(kAW * 32) r_barp(AArgs A, const double* gT, const double* hT, const double* mC,
                                                   const double* lgB, const double* lhB, double* lgT, double* lhT,
                                                   double* lm) {
    using SJ = ShakhovJacT<D>;
    extern __shared__ double eTab[];
    const StepArgs& a = A.a;
    const int lane = threadIdx.x & 31, Vp = a.Vp, M = A.M;
    double* E = eTab + (threadIdx.x >> 5) * D * M;
    for (int c = blockIdx.x * kAW + (threadIdx.x >> 5); c < a.nC; c += gridDim.x * kAW) {
        const long long base = (long long)c * Vp;
        const double* m = mC + (size_t)kM * c;
        const double r = 1.5 * a.dt / (2.0 * m[8] + a.dt);
        const double dr = -3.0 * a.dt / ((2.0 * m[8] + a.dt) * (2.0 * m[8] + a.dt));
        SJ J;
        J.prep(m, a.R, a.Pr, a.K);
        gauss_table<D>(a, M, J.U, J.ith, E);
        double acc[SJ::NJ];
#pragma unroll
        for (int i = 0; i < SJ::NJ; ++i) acc[i] = 0.0;
        DvIdx<D> id;
        id.init(lane, M);
        for (int v = lane; v < a.nV; v += 32, id.advance(32, M)) {
            double x[D], cv[D], cc = 0.0;
            load_xi<D>(a, v, x);
#pragma unroll
            for (int k = 0; k < D; ++k) { cv[k] = x[k] - J.U[k]; cc += cv[k] * cv[k]; }
            double G0 = J.N * E[id.ix] * E[M + id.iy];
            if (D == 3) G0 *= E[2 * M + id.iz];
            const double lg = lgB[base + v], lh = HH ? lhB[base + v] : 0.0;
            J.apply(cv, cc, G0, gT[base + v], HH ? hT[base + v] : 0.0, lg, lh, acc);
            lgT[base + v] += (1.0 - r) * lg;
            if (HH) lhT[base + v] += (1.0 - r) * lh;
        }
        wsum<SJ::NJ>(acc);
        double out[kM];
        J.finish(acc, r, dr, a.R, out);
        if (lane == 0)
#pragma unroll
            for (int k = 0; k < kM; ++k) lm[(size_t)kM * c + k] = out[k];
    }
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

namespace {
int wgrid(int n, int sms) {  // blocks of kAW warps, one warp per entity, grid-stride
    const long long b = ((long long)n + kAW - 1) / kAW, cap = (long long)sms * 16;
    return (int)(b < cap ? (b > 0 ? b : 1) : cap);
}

template <int D, bool HH>
void adj_step(const AdjState& s, const double* gTn, const double* hTn, const double* mTn, bool objective,
              double scale, int sms, cudaStream_t st) {
    const AArgs A{s.a, s.a.Tw, s.muRef, s.M};
    const StepArgs& a = s.a;
    const size_t eTab = (size_t)kAW * D * s.M * sizeof(double);
    const int gC = wgrid(a.nC, sms), gF = wgrid(a.nA, sms), thr = kAW * 32;
    // P9 reverse fused with the cell part of P8 (lgN += J9^T lmN; lgT, lgB from lgN)
    if (s.haveMacroAdj)
        r_cell_mom<D, HH><<<gC, thr, 0, st>>>(A, gTn, hTn, mTn, s.lgN, s.lhN, s.lgT, s.lhT, s.lgB, s.lhB, s.lmN,
                                             s.lmuC);
    else
        r_cell_flux<<<grid((long long)a.nC * a.Vp, kT, sms), kT, 0, st>>>(A, s.lgN, s.lhN, s.lgT, s.lhT, s.lgB,
                                                                           s.lhB);
    // P8 reverse, face part
    r_face_flux<D, HH><<<gF, thr, 0, st>>>(A, s.lgN, s.lhN, s.lgS, s.lhS);
    // P7 + P6 reverse
    r_face<D, HH><<<gF, thr, eTab, st>>>(A, s.gS, s.hS, s.mF, s.lgS, s.lhS, s.wq, s.ws, objective ? scale : 0.0,
                                         s.lmuF);
    // P5 + P4 reverse
    if (a.nW > 0) r_wall<<<a.nW, kRT, 0, st>>>(A, s.gS, a.rhoW, a.incAbs, s.lgS, s.lhS, s.lTw);
    // P3 reverse (+ G_b' = grad.n), P2 reverse
    r_recon<D, HH><<<gC, thr, 0, st>>>(A, s.lgS, s.lhS, s.lGbN, s.lGbNh, s.lgB, s.lhB, s.lG, s.lhG);
    r_grad<D, HH><<<gC, thr, 0, st>>>(A, s.lG, s.lhG, s.lgB, s.lhB, s.lGb, s.lGbh);
    // P1 reverse
    r_barp<D, HH><<<gC, thr, eTab, st>>>(A, s.gT, s.hT, s.mC, s.lgB, s.lhB, s.lgT, s.lhT, s.lm);
}
}  // namespace

size_t adj_table_bytes(int D, int M) { return (size_t)kAW * D * M * sizeof(double); }

void adj_launch_step(const AdjState& s, const double* gTn, const double* hTn, const double* mTn, bool objective,
                     double scale, int sms, cudaStream_t st) {
    if (s.a.D == 3) {
        if (s.a.hasH) adj_step<3, true>(s, gTn, hTn, mTn, objective, scale, sms, st);
        else adj_step<3, false>(s, gTn, hTn, mTn, objective, scale, sms, st);
    } else {
        adj_step<2, true>(s, gTn, hTn, mTn, objective, scale, sms, st);
    }
}

void adj_sum(int n, const double* x, double* out, cudaStream_t st) { k_sum<<<1, kT, 0, st>>>(n, x, out); }

}  // namespace dugks
