// Reference pipeline: one FP64 kernel per pass of fvDVM::evolution()
// (src/fvDVM/fvDVM/fvDVM.C:1086-1108), with every intermediate materialised
// in HBM (DV index innermost).  It is the plain, easily checked GPU
// restatement; the fused tile sweeps (fused_pipeline.cu) are the fast path.
//
//   k_barp      P1 updateGHbarPvol             discreteVelocity.C:346-410
//   k_grad      P2 fvc::grad + fixedGradient   discreteVelocity.C:420-470
//   k_recon     P3 updateGHbarSurf             discreteVelocity.C:472-691
//   k_wall      P4+P5 MaxwellWallRho / WallIn  fvDVM.C:347-367, discreteVelocity.C:693-731
//   k_sym_*     P5b updateGHbarSurfSymmetryIn  fvDVM.C:375-454, discreteVelocity.C:733-817
//   k_face_mom  P6 updateMacroSurf             fvDVM.C:456-582
//   k_relax     P7 updateGHsurf                discreteVelocity.C:819-932
//   k_cell      P8 updateGHtildeVol            discreteVelocity.C:934-978
//   k_cell_mom  P9 updateMacroVol              fvDVM.C:597-728
//   k_pressure  P10 updatePressureInOutBC      fvDVM.C:730-806
//
// Boundary faces follow the surface patch type of their rho boundary
// condition (discreteVelocity::setBCtype, discreteVelocity.C:250-300):
// diffuse walls, zeroGradient, mixed (rho fixedValue), farField (also for
// pressureIn / pressureOut) and the two symmetry types.
#include "device_common.cuh"
#include "kernels.h"

namespace dugks {
namespace {

constexpr int kThreads = 256;
constexpr int kRedThreads = 128;

__device__ __forceinline__ void dv_index(long long i, int Vp, int& e, int& v) {
    e = (int)(i / Vp);
    v = (int)(i - (long long)e * Vp);
}

__global__ void k_barp(StepArgs a, const double* __restrict__ gT, const double* __restrict__ hT,
                       double* __restrict__ gB, double* __restrict__ hB) {
    const long long n = (long long)a.nC * a.Vp;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        int c, v;
        dv_index(i, a.Vp, c, v);
        if (v >= a.nV) continue;
        const double dt = a.dt;
        double rf = 1.5 * dt / (2.0 * a.tau[c] + dt);
        double ge, he;
        shakhov_ref(a.rho[c], a.U[3 * c], a.U[3 * c + 1], a.U[3 * c + 2], a.T[c], a.q[3 * c], a.q[3 * c + 1],
                    a.q[3 * c + 2], a.xi[v], a.xi[a.Vp + v], a.xi[2 * a.Vp + v], a.R, a.Pr, a.D, a.K, ge, he);
        gB[i] = (1.0 - rf) * gT[i] + rf * ge;
        if (a.hasH) hB[i] = (1.0 - rf) * hT[i] + rf * he;
    }
}

// Least-squares gradient of gBarPvol (cell-centric gather in increasing face
// order = the reference's scatter order), fixedGradient boundary value
// phi_b = phi_P + G_b/deltaCoeff_b with the lagged G_b, then G_b <- grad.n.
__global__ void k_grad(StepArgs a, const double* __restrict__ gB, const double* __restrict__ hB,
                       double* __restrict__ gG, double* __restrict__ hG, double* __restrict__ Gbg,
                       double* __restrict__ Gbh) {
    const long long n = (long long)a.nC * a.Vp;
    const int D = a.D, Vp = a.Vp;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        int c, v;
        dv_index(i, Vp, c, v);
        if (v >= a.nV) continue;
        double g[3] = {0, 0, 0}, h[3] = {0, 0, 0};
        const double gc = gB[i];
        const double hc = a.hasH ? hB[i] : 0.0;
        for (int j = a.cellOff[c]; j < a.cellOff[c + 1]; ++j) {
            int e = a.cellFace[j], f = chk(e >> 1, a.nA, a.status), side = e & 1;
            if (f < a.nI) {
                int o = chk(a.own[f], a.nC, a.status), nb = chk(a.nei[f], a.nC, a.status);
                double dg = gB[(long long)nb * Vp + v] - gB[(long long)o * Vp + v];
                double dh = a.hasH ? hB[(long long)nb * Vp + v] - hB[(long long)o * Vp + v] : 0.0;
                const double* L = side ? a.nVec + 3 * f : a.pVec + 3 * f;
                if (side == 0) {
                    for (int k = 0; k < D; ++k) { g[k] += L[k] * dg; h[k] += L[k] * dh; }
                } else {
                    for (int k = 0; k < D; ++k) { g[k] -= L[k] * dg; h[k] -= L[k] * dh; }
                }
            } else {
                int wf = f - a.nI;
                long long wi = (long long)wf * Vp + v;
                // symmetryPlane is a constraint patch of gBarPvol: its scalar
                // value is the internal value, so it adds nothing
                const bool sym = a.bKind[wf] == kBcSymmetryPlane;
                double gbv = sym ? gc : gc + Gbg[wi] / a.dcW[wf];
                double dg = gbv - gc;
                double dh = 0.0;
                if (a.hasH) { double hbv = sym ? hc : hc + Gbh[wi] / a.dcW[wf]; dh = hbv - hc; }
                const double* L = a.bVec + 3 * wf;
                for (int k = 0; k < D; ++k) { g[k] += L[k] * dg; h[k] += L[k] * dh; }
            }
        }
        for (int k = 0; k < D; ++k) {
            gG[((long long)c * D + k) * Vp + v] = g[k];
            if (a.hasH) hG[((long long)c * D + k) * Vp + v] = h[k];
        }
        for (int j = a.cellOff[c]; j < a.cellOff[c + 1]; ++j) {
            int f = chk(a.cellFace[j] >> 1, a.nA, a.status);
            if (f < a.nI) continue;
            int wf = f - a.nI;
            const double* nh = a.nHatW + 3 * wf;
            double sg = 0.0, sh = 0.0;
            for (int k = 0; k < D; ++k) { sg += g[k] * nh[k]; sh += h[k] * nh[k]; }
            Gbg[(long long)wf * Vp + v] = sg;
            if (a.hasH) Gbh[(long long)wf * Vp + v] = sh;
        }
    }
}

__device__ __forceinline__ double recon(const double* __restrict__ f, const double* __restrict__ G, long long c,
                                        int v, int Vp, int D, const double* d, const double* xi, double dt) {
    double s = f[c * Vp + v];
    double acc = 0.0;
    for (int k = 0; k < D; ++k) acc += G[(c * D + k) * Vp + v] * (d[k] - 0.5 * xi[k] * dt);
    return s + acc;
}

__global__ void k_recon(StepArgs a, const double* __restrict__ gB, const double* __restrict__ hB,
                        const double* __restrict__ gG, const double* __restrict__ hG, double* __restrict__ gS,
                        double* __restrict__ hS) {
    const long long n = (long long)a.nA * a.Vp;
    const int D = a.D, Vp = a.Vp;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        int f, v;
        dv_index(i, Vp, f, v);
        if (v >= a.nV) continue;
        double xi[3] = {a.xi[v], a.xi[Vp + v], a.xi[2 * Vp + v]};
        const double* S = a.Sf + 3 * f;
        double xs = xi[0] * S[0] + xi[1] * S[1] + xi[2] * S[2];
        const double* dO = a.dO + 3 * f;
        if (f < a.nI) {
            const double* dN = a.dN + 3 * f;
            int o = chk(a.own[f], a.nC, a.status), nb = chk(a.nei[f], a.nC, a.status);
            if (xs >= kVSmall) {
                gS[i] = recon(gB, gG, o, v, Vp, D, dO, xi, a.dt);
                if (a.hasH) hS[i] = recon(hB, hG, o, v, Vp, D, dO, xi, a.dt);
            } else if (xs < -kVSmall) {
                gS[i] = recon(gB, gG, nb, v, Vp, D, dN, xi, a.dt);
                if (a.hasH) hS[i] = recon(hB, hG, nb, v, Vp, D, dN, xi, a.dt);
            } else {
                gS[i] = 0.5 * (recon(gB, gG, nb, v, Vp, D, dN, xi, a.dt) + recon(gB, gG, o, v, Vp, D, dO, xi, a.dt));
                if (a.hasH)
                    hS[i] = 0.5 * (recon(hB, hG, nb, v, Vp, D, dN, xi, a.dt) + recon(hB, hG, o, v, Vp, D, dO, xi, a.dt));
            }
        } else {
            const int wf = f - a.nI, kind = a.bKind[wf], o = chk(a.own[f], a.nC, a.status);
            if (kind == kBcZeroGradient) {  // gSurf == gBarPvol patchInternalField, every DV
                gS[i] = gB[(long long)o * Vp + v];
                if (a.hasH) hS[i] = hB[(long long)o * Vp + v];
                continue;
            }
            const bool sym = kind == kBcSymmetryMod || kind == kBcSymmetryPlane;
            if (sym ? xs > -kVSmall : xs > 0) {  // outgoing (and tangential on symmetry patches)
                gS[i] = recon(gB, gG, o, v, Vp, D, dO, xi, a.dt);
                if (a.hasH) hS[i] = recon(hB, hG, o, v, Vp, D, dO, xi, a.dt);
            } else if (kind == kBcFarField || kind == kBcPressureIn || kind == kBcPressureOut) {
                // incoming: rho_b M(U of the owner cell, T_b) (discreteVelocity.C:570-600)
                const double Tb = a.TbM[wf];
                const double g = a.rhoB[wf] * maxwell_by_rho_ref(a.U[3 * o], a.U[3 * o + 1], a.U[3 * o + 2], Tb,
                                                                 xi[0], xi[1], xi[2], a.R, a.D);
                gS[i] = g;
                if (a.hasH) hS[i] = g * (a.R * Tb) * (a.K + 3 - a.D);
            }
        }
    }
}

// One block per wall face: rho_w = sum_out w (xi.S) gbar / |inComingByRho|,
// then incoming DVs (xi.S <= 0) get rho_w * Maxwellian(U_w, T_w).
__global__ void k_wall(StepArgs a, double* __restrict__ gS, double* __restrict__ hS) {
    __shared__ double red[32];
    const int wf = blockIdx.x;
    if (a.bKind[wf] != kBcMaxwell) return;  // uniform over the block
    const int f = a.nI + wf;
    const int Vp = a.Vp;
    const double* S = a.Sf + 3 * f;
    double acc[1] = {0.0};
    for (int v = threadIdx.x; v < a.nV; v += blockDim.x) {
        double xs = a.xi[v] * S[0] + a.xi[Vp + v] * S[1] + a.xi[2 * Vp + v] * S[2];
        if (xs > 0) acc[0] += a.w[v] * xs * gS[(long long)f * Vp + v];
    }
    block_sum<1>(acc, red);
    const double rw = acc[0] / a.incAbs[wf];
    if (threadIdx.x == 0) a.rhoW[wf] = rw;
    const double Tw = a.Tw[wf];
    const double* Uw = a.Uw + 3 * wf;
    for (int v = threadIdx.x; v < a.nV; v += blockDim.x) {
        double x0 = a.xi[v], x1 = a.xi[Vp + v], x2 = a.xi[2 * Vp + v];
        double xs = x0 * S[0] + x1 * S[1] + x2 * S[2];
        if (xs <= 0) {
            double g = rw * maxwell_by_rho_ref(Uw[0], Uw[1], Uw[2], Tw, x0, x1, x2, a.R, a.D);
            gS[(long long)f * Vp + v] = g;
            if (a.hasH) hS[(long long)f * Vp + v] = g * (a.R * Tw) * (a.K + 3 - a.D);
        }
    }
}

// Symmetry patches, step 1: snapshot of the face values of every velocity.
__global__ void k_sym_snap(StepArgs a, const double* __restrict__ gS, const double* __restrict__ hS,
                           double* __restrict__ gSnap, double* __restrict__ hSnap) {
    const int wf = blockIdx.x;
    if (a.symOff[wf] < 0) return;
    const long long fb = (long long)(a.nI + wf) * a.Vp, wb = (long long)wf * a.Vp;
    for (int v = threadIdx.x; v < a.nV; v += blockDim.x) {
        gSnap[wb + v] = gS[fb + v];
        if (a.hasH) hSnap[wb + v] = hS[fb + v];
    }
}

// Step 2: incoming velocities (xi.S0 <= 0, S0 the patch's first face) take
// their mirror velocity's value.  DVMsymmetry reads the snapshot; symmetryPlane
// assigns velocity by velocity in index order, so a mirror that is itself an
// earlier incoming velocity already holds its own mirror's value: the chain is
// followed back to a snapshot value (one step on grids symmetric about 0).
__global__ void k_sym_in(StepArgs a, double* __restrict__ gS, double* __restrict__ hS,
                         const double* __restrict__ gSnap, const double* __restrict__ hSnap) {
    const int wf = blockIdx.x;
    const int row = a.symOff[wf];
    if (row < 0) return;
    const int Vp = a.Vp, nV = a.nV;
    const bool plane = a.bKind[wf] == kBcSymmetryPlane;
    const double* S0 = a.bS0 + 3 * wf;
    const int* tab = a.symTab + (long long)row * nV;
    const long long fb = (long long)(a.nI + wf) * Vp, wb = (long long)wf * Vp;
    auto incoming = [&](int u) { return a.xi[u] * S0[0] + a.xi[Vp + u] * S0[1] + a.xi[2 * Vp + u] * S0[2] <= 0; };
    for (int v = threadIdx.x; v < nV; v += blockDim.x) {
        if (!incoming(v)) continue;
        int cur = v, u = tab[v];
        if (plane)
            for (int guard = 0; guard < nV && u < cur && incoming(u); ++guard) {
                cur = u;
                u = tab[u];
            }
        gS[fb + v] = gSnap[wb + u];
        if (a.hasH) hS[fb + v] = hSnap[wb + u];
    }
}

// One block per active face: face macros (two DV passes as the reference),
// plus qWall / stressWall on wall faces.
__global__ void k_face_mom(StepArgs a, const double* __restrict__ gS, const double* __restrict__ hS) {
    __shared__ double red[32 * 12];
    const int f = blockIdx.x;
    const int Vp = a.Vp;
    const long long base = (long long)f * Vp;
    double m[5] = {0, 0, 0, 0, 0};
    for (int v = threadIdx.x; v < a.nV; v += blockDim.x) {
        double x0 = a.xi[v], x1 = a.xi[Vp + v], x2 = a.xi[2 * Vp + v], w = a.w[v];
        double g = gS[base + v], h = a.hasH ? hS[base + v] : 0.0;
        m[0] += w * g;
        m[1] += w * g * x0;
        m[2] += w * g * x1;
        m[3] += w * g * x2;
        m[4] += 0.5 * w * (g * (x0 * x0 + x1 * x1 + x2 * x2) + h);
    }
    block_sum<5>(m, red);
    const double rho = m[0];
    const double Ux = m[1] / rho, Uy = m[2] / rho, Uz = m[3] / rho;
    const double T = (m[4] - 0.5 * rho * (Ux * Ux + Uy * Uy + Uz * Uz)) / ((a.K + 3) / 2.0 * a.R * rho);
    const double tau = tau_ref(T, rho, a.muRef, a.omega, a.Tref, a.R);
    const int wf = f - a.nI;
    const bool wall = f >= a.nI && a.bKind[wf] == kBcMaxwell;
    double qq[15];
    for (int i = 0; i < 15; ++i) qq[i] = 0.0;
    double Uw0 = 0, Uw1 = 0, Uw2 = 0;
    if (wall) { Uw0 = a.Uw[3 * wf]; Uw1 = a.Uw[3 * wf + 1]; Uw2 = a.Uw[3 * wf + 2]; }
    for (int v = threadIdx.x; v < a.nV; v += blockDim.x) {
        double x0 = a.xi[v], x1 = a.xi[Vp + v], x2 = a.xi[2 * Vp + v], w = a.w[v];
        double g = gS[base + v], h = a.hasH ? hS[base + v] : 0.0;
        double c0 = x0 - Ux, c1 = x1 - Uy, c2 = x2 - Uz;
        double s = (c0 * c0 + c1 * c1 + c2 * c2) * g + h;
        qq[0] += 0.5 * w * c0 * s;
        qq[1] += 0.5 * w * c1 * s;
        qq[2] += 0.5 * w * c2 * s;
        if (wall) {
            double e0 = x0 - Uw0, e1 = x1 - Uw1, e2 = x2 - Uw2;
            double sw = (e0 * e0 + e1 * e1 + e2 * e2) * g + h;
            qq[3] += 0.5 * 1.0 * w * e0 * sw;
            qq[4] += 0.5 * 1.0 * w * e1 * sw;
            qq[5] += 0.5 * 1.0 * w * e2 * sw;
            double wg = 1.0 * w * g;
            qq[6] += wg * x0 * x0; qq[7] += wg * x0 * x1; qq[8] += wg * x0 * x2;
            qq[9] += wg * x1 * x0; qq[10] += wg * x1 * x1; qq[11] += wg * x1 * x2;
            qq[12] += wg * x2 * x0; qq[13] += wg * x2 * x1; qq[14] += wg * x2 * x2;
        }
    }
    if (wall) {
        block_sum<15>(qq, red);
    } else {
        double q3[3] = {qq[0], qq[1], qq[2]};
        block_sum<3>(q3, red);
        qq[0] = q3[0]; qq[1] = q3[1]; qq[2] = q3[2];
    }
    if (threadIdx.x == 0) {
        const double dt = a.dt;
        a.rhoF[f] = rho;
        a.UF[3 * f] = Ux; a.UF[3 * f + 1] = Uy; a.UF[3 * f + 2] = Uz;
        a.TF[f] = T;
        a.tauF[f] = tau;
        double fac = 2.0 * tau / (2.0 * tau + 0.5 * dt * a.Pr);
        a.qF[3 * f] = fac * qq[0]; a.qF[3 * f + 1] = fac * qq[1]; a.qF[3 * f + 2] = fac * qq[2];
        if (wall) {
            double fq = 2.0 * tau / (2.0 * tau + 0.5 * dt * a.Pr);
            double fs = 2.0 * tau / (2.0 * tau + 0.5 * dt);
            for (int k = 0; k < 3; ++k) a.qWall[3 * wf + k] = fq * qq[3 + k];
            for (int k = 0; k < 9; ++k) a.stressWall[9 * wf + k] = fs * qq[6 + k];
        }
    }
}

__global__ void k_relax(StepArgs a, double* __restrict__ gS, double* __restrict__ hS) {
    const long long n = (long long)a.nA * a.Vp;
    const int Vp = a.Vp;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        int f, v;
        dv_index(i, Vp, f, v);
        if (v >= a.nV) continue;
        double x0 = a.xi[v], x1 = a.xi[Vp + v], x2 = a.xi[2 * Vp + v];
        int times = 1;
        if (f >= a.nI) {
            // The project's surface patch types ignore the field assignment
            // (e.g. maxwellWallFvsPatchField.H:163-181), symmetryPlane takes it;
            // then every outgoing DV is relaxed once more (discreteVelocity.C:887-931).
            const double* S = a.Sf + 3 * f;
            times = (a.bKind[f - a.nI] == kBcSymmetryPlane) + (x0 * S[0] + x1 * S[1] + x2 * S[2] > 0);
            if (times == 0) continue;  // incoming boundary DVs stay unrelaxed
        }
        const double hh = 0.5 * a.dt;
        double b = hh / (2 * a.tauF[f] + hh);
        double ge, he;
        shakhov_ref(a.rhoF[f], a.UF[3 * f], a.UF[3 * f + 1], a.UF[3 * f + 2], a.TF[f], a.qF[3 * f], a.qF[3 * f + 1],
                    a.qF[3 * f + 2], x0, x1, x2, a.R, a.Pr, a.D, a.K, ge, he);
        for (int t = 0; t < times; ++t) {
            gS[i] = (1.0 - b) * gS[i] + b * ge;
            if (a.hasH) hS[i] = (1.0 - b) * hS[i] + b * he;
        }
    }
}

__global__ void k_cell(StepArgs a, double* __restrict__ gT, double* __restrict__ hT, const double* __restrict__ gB,
                       const double* __restrict__ hB, const double* __restrict__ gS, const double* __restrict__ hS) {
    const long long n = (long long)a.nC * a.Vp;
    const int Vp = a.Vp;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        int c, v;
        dv_index(i, Vp, c, v);
        if (v >= a.nV) continue;
        double x0 = a.xi[v], x1 = a.xi[Vp + v], x2 = a.xi[2 * Vp + v];
        const double dt = a.dt, V = a.vol[c];
        double g = -1.0 / 3 * gT[i] + 4.0 / 3 * gB[i];
        double h = a.hasH ? -1.0 / 3 * hT[i] + 4.0 / 3 * hB[i] : 0.0;
        for (int j = a.cellOff[c]; j < a.cellOff[c + 1]; ++j) {
            int e = a.cellFace[j], f = chk(e >> 1, a.nA, a.status);
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

__global__ void k_cell_mom(StepArgs a, const double* __restrict__ gT, const double* __restrict__ hT) {
    __shared__ double red[32 * 5];
    const int c = blockIdx.x;
    const int Vp = a.Vp;
    const long long base = (long long)c * Vp;
    double m[5] = {0, 0, 0, 0, 0};
    for (int v = threadIdx.x; v < a.nV; v += blockDim.x) {
        double x0 = a.xi[v], x1 = a.xi[Vp + v], x2 = a.xi[2 * Vp + v], w = a.w[v];
        double g = gT[base + v], h = a.hasH ? hT[base + v] : 0.0;
        m[0] += w * g;
        m[1] += w * g * x0;
        m[2] += w * g * x1;
        m[3] += w * g * x2;
        m[4] += 0.5 * w * ((x0 * x0 + x1 * x1 + x2 * x2) * g + h);
    }
    block_sum<5>(m, red);
    const double rho = m[0];
    const double Ux = m[1] / rho, Uy = m[2] / rho, Uz = m[3] / rho;
    const double T = (m[4] - 0.5 * rho * (Ux * Ux + Uy * Uy + Uz * Uz)) / ((a.K + 3) / 2.0 * a.R * rho);
    const double tau = tau_ref(T, rho, a.muRef, a.omega, a.Tref, a.R);
    double qq[3] = {0, 0, 0};
    for (int v = threadIdx.x; v < a.nV; v += blockDim.x) {
        double x0 = a.xi[v], x1 = a.xi[Vp + v], x2 = a.xi[2 * Vp + v], w = a.w[v];
        double g = gT[base + v], h = a.hasH ? hT[base + v] : 0.0;
        double c0 = x0 - Ux, c1 = x1 - Uy, c2 = x2 - Uz;
        double s = (c0 * c0 + c1 * c1 + c2 * c2) * g + h;
        qq[0] += 0.5 * w * c0 * s;
        qq[1] += 0.5 * w * c1 * s;
        qq[2] += 0.5 * w * c2 * s;
    }
    block_sum<3>(qq, red);
    if (threadIdx.x == 0) {
        a.rho[c] = rho;
        a.U[3 * c] = Ux; a.U[3 * c + 1] = Uy; a.U[3 * c + 2] = Uz;
        a.T[c] = T;
        a.tau[c] = tau;
        double fac = 2.0 * tau / (2.0 * tau + a.dt * a.Pr);
        a.q[3 * c] = fac * qq[0]; a.q[3 * c + 1] = fac * qq[1]; a.q[3 * c + 2] = fac * qq[2];
        if (!(rho > 0.0) || !(T > 0.0) || !isfinite(Ux + Uy + Uz + qq[0] + qq[1] + qq[2])) atomicExch(a.status, 5);
    }
}

// P10: pressureIn / pressureOut patch values from the new cell macros of the
// owner (characteristic relations of fvDVM::updatePressureInOutBC).
__global__ void k_pressure(StepArgs a) {
    const int wf = blockIdx.x * blockDim.x + threadIdx.x;
    if (wf >= a.nW) return;
    const int kind = a.bKind[wf];
    if (kind != kBcPressureIn && kind != kBcPressureOut) return;
    const int f = a.nI + wf, P = a.own[f];
    const double* Sf = a.Sf + 3 * f;
    const double magSf = sqrt(Sf[0] * Sf[0] + Sf[1] * Sf[1] + Sf[2] * Sf[2]);
    const double n[3] = {Sf[0] / magSf, Sf[1] / magSf, Sf[2] / magSf};
    const double Ui[3] = {a.U[3 * P], a.U[3 * P + 1], a.U[3 * P + 2]};
    const double Ti = a.T[P], rhoi = a.rho[P], R = a.R, p = a.pB[wf];
    const double ai = sqrt(R * Ti * (a.K + 5) / (a.K + 3));
    const double Un = Ui[0] * n[0] + Ui[1] * n[1] + Ui[2] * n[2];
    double UnIn;
    if (kind == kBcPressureIn) {
        a.rhoB[wf] = p / R / a.TbM[wf];
        UnIn = Un + (p - rhoi * R * Ti) / rhoi / ai;
    } else {
        a.rhoB[wf] = rhoi + (p - rhoi * R * Ti) / ai / ai;
        a.TbM[wf] = p / (R * rhoi);
        UnIn = Un + (rhoi * R * Ti - p) / rhoi / ai;
    }
    for (int k = 0; k < 3; ++k) a.UbM[3 * wf + k] = UnIn * n[k] + (Ui[k] - Un * n[k]);
}

// Uvol_/Tvol_.correctBoundaryConditions() (fvDVM.C:697-699) after the cell
// macros: a zeroGradient U or T patch takes its owner cell's new value (before
// P10, which reads T_b on pressureIn patches).
__global__ void k_zero_gradient_tu(StepArgs a) {
    const int wf = blockIdx.x * blockDim.x + threadIdx.x;
    if (wf >= a.nW) return;
    const int zg = a.bZG[wf];
    if (!zg) return;
    const int P = a.own[a.nI + wf];
    if (zg & 1) a.TbM[wf] = a.T[P];
    if (zg & 2)
        for (int k = 0; k < 3; ++k) a.UbM[3 * wf + k] = a.U[3 * P + k];
}

// Initial face values of mixed patches (rho fixedValue): the Maxwellian of the
// patch rho, U, T for every DV (discreteVelocity::initBoundaryField,
// discreteVelocity.C:302-345, equilibriumMaxwell :1046-1061).
__global__ void k_mixed_init(StepArgs a, double* __restrict__ gS, double* __restrict__ hS) {
    const int wf = blockIdx.x;
    if (a.bKind[wf] != kBcFixedValue) return;
    const long long fb = (long long)(a.nI + wf) * a.Vp;
    const double rho = a.rhoB[wf], T = a.TbM[wf], R = a.R;
    const double* U = a.UbM + 3 * wf;
    const double s = sqrt(2.0 * kPi * R * T);
    const double pw = (a.D == 2) ? s * s : (a.D == 3 ? s * s * s : s);
    for (int v = threadIdx.x; v < a.nV; v += blockDim.x) {
        const double c0 = U[0] - a.xi[v], c1 = U[1] - a.xi[a.Vp + v], c2 = U[2] - a.xi[2 * a.Vp + v];
        const double g = rho / pw * exp(-(c0 * c0 + c1 * c1 + c2 * c2) / (2.0 * R * T));
        gS[fb + v] = g;
        if (a.hasH) hS[fb + v] = (a.K + 3 - a.D) * R * T * g;
    }
}

int grid_for(long long n, int threads, int sms) {
    long long b = (n + threads - 1) / threads;
    long long cap = (long long)sms * 32;
    return (int)(b < cap ? (b > 0 ? b : 1) : cap);
}

}  // namespace

void launch_pressure_bc(const StepArgs& a, cudaStream_t s) {
    if (a.nW > 0) k_pressure<<<(a.nW + 127) / 128, 128, 0, s>>>(a);
}

void launch_zero_gradient_tu(const StepArgs& a, cudaStream_t s) {
    if (a.nW > 0 && a.zgMask) k_zero_gradient_tu<<<(a.nW + 127) / 128, 128, 0, s>>>(a);
}

void launch_ref_mixed_init(const StepArgs& a, const RefBuffers& b, cudaStream_t s) {
    if (a.nW > 0 && (a.bcMask & (1 << kBcFixedValue))) k_mixed_init<<<a.nW, kRedThreads, 0, s>>>(a, b.gS, b.hS);
}

const char* const kRefKernelNames[kRefKernels] = {"k_barp", "k_grad", "k_recon", "k_wall",
                                                  "k_face_mom", "k_relax", "k_cell", "k_cell_mom"};

void launch_ref_pass(int pass, const StepArgs& a, const RefBuffers& b, int sms, cudaStream_t s) {
    const long long nCV = (long long)a.nC * a.Vp, nAV = (long long)a.nA * a.Vp;
    switch (pass) {
        case 0: k_barp<<<grid_for(nCV, kThreads, sms), kThreads, 0, s>>>(a, b.gT, b.hT, b.gB, b.hB); break;
        case 1: k_grad<<<grid_for(nCV, kThreads, sms), kThreads, 0, s>>>(a, b.gB, b.hB, b.gG, b.hG, b.Gbg, b.Gbh); break;
        case 2: k_recon<<<grid_for(nAV, kThreads, sms), kThreads, 0, s>>>(a, b.gB, b.hB, b.gG, b.hG, b.gS, b.hS); break;
        case 3:
            if (a.nW > 0 && (a.bcMask & (1 << kBcMaxwell))) k_wall<<<a.nW, kRedThreads, 0, s>>>(a, b.gS, b.hS);
            if (a.bcMask & ((1 << kBcSymmetryMod) | (1 << kBcSymmetryPlane))) {
                k_sym_snap<<<a.nW, kRedThreads, 0, s>>>(a, b.gS, b.hS, b.gSym, b.hSym);
                k_sym_in<<<a.nW, kRedThreads, 0, s>>>(a, b.gS, b.hS, b.gSym, b.hSym);
            }
            break;
        case 4: k_face_mom<<<a.nA, kRedThreads, 0, s>>>(a, b.gS, b.hS); break;
        case 5: k_relax<<<grid_for(nAV, kThreads, sms), kThreads, 0, s>>>(a, b.gS, b.hS); break;
        case 6: k_cell<<<grid_for(nCV, kThreads, sms), kThreads, 0, s>>>(a, b.gT, b.hT, b.gB, b.hB, b.gS, b.hS); break;
        case 7:
            k_cell_mom<<<a.nC, kRedThreads, 0, s>>>(a, b.gT, b.hT);
            if (a.zgMask) k_zero_gradient_tu<<<(a.nW + 127) / 128, 128, 0, s>>>(a);
            if (a.bcMask & ((1 << kBcPressureIn) | (1 << kBcPressureOut)))
                k_pressure<<<(a.nW + 127) / 128, 128, 0, s>>>(a);
            break;
        default: break;
    }
}

}  // namespace dugks
