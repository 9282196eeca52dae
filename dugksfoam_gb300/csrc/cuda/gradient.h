// Differentiated FP64 step (gradient.cu): device state of the tangent-linear
// and adjoint sweeps, and their launchers.
#pragma once

#include <cuda_runtime.h>

#include "device_common.cuh"
#include "dual.cuh"

namespace dugks {

// Tangent-linear state: the reference-pipeline buffers and macros as Dual.
struct TlmState {
    StepArgs a;  // geometry, DV set, dt, gas; macro pointers unused
    Dual *gT, *hT, *gB, *hB, *gG, *hG, *Gbg, *Gbh, *gS, *hS;
    Dual *rho, *U, *T, *q, *tau;
    Dual *rhoF, *UF, *TF, *qF, *tauF;
    Dual *rhoW, *qWall, *stressWall;
    Dual *Tw, *incAbs;
    Dual muRef;
};

// Adjoint state of one reverse step n (forward intermediates of step n in
// `a` and the pointers below; adjoint buffers).
struct AdjState {
    StepArgs a;                 // forward arguments (macros of the recomputed step)
    double muRef;
    const double *gT, *hT;      // state n
    const double *gS, *hS;      // face values of step n before relaxation
    const double* mC;           // [nC][9] cell macros at the start of step n
    const double* mF;           // [nA][9] face macros of step n
    const double *wq, *ws;      // objective weights per wall face
    double *lgN, *lhN;          // in: adjoint of state n+1 (modified)
    double *lgT, *lhT;          // out: adjoint of state n
    double *lgB, *lhB, *lG, *lhG, *lgS, *lhS;
    double *lGbN, *lGbNh;       // in: adjoint of the lagged wall gradient G_b(n+1)
    double *lGb, *lGbh;         // out: adjoint of G_b(n)
    const double* lmN;          // in: adjoint of the cell macros at n+1 ([nC][9])
    double* lm;                 // out: adjoint of the cell macros at n
    bool haveMacroAdj;          // lmN is nonzero
    int M;                      // velocities per direction of the tensor-product grid
    double *lmuC, *lmuF, *lTw;  // accumulated parameter adjoints
};

void tlm_launch_incabs(const TlmState& s, cudaStream_t st);
void tlm_launch_init(const TlmState& s, const double* rho0, const double* U0, const double* T0, int sms,
                     cudaStream_t st);
void tlm_launch_step(const TlmState& s, bool objective, const double* wq, const double* ws, double scale, Dual* J,
                     int sms, cudaStream_t st);

void launch_objective(const StepArgs& a, const double* wq, const double* ws, double scale, double* J, cudaStream_t st);
void adj_pack_macros(int n, const double* rho, const double* U, const double* T, const double* q, const double* tau,
                     double* out, int sms, cudaStream_t st);
// One reverse step.  gTn, hTn: state n+1; mTn: its cell macros as stored
// (rho [nC], U [nC][3], T [nC], q [nC][3], tau [nC]).  2D cases carry h
// (K + 3 - D > 0); 3D cases with or without it.
void adj_launch_step(const AdjState& s, const double* gTn, const double* hTn, const double* mTn, bool objective,
                     double scale, int sms, cudaStream_t st);
// Shared memory of the per-warp Gaussian tables (must stay within 48 KB).
size_t adj_table_bytes(int D, int M);
void adj_sum(int n, const double* x, double* out, cudaStream_t st);

}  // namespace dugks
