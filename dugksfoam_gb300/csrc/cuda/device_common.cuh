// Device-side helpers shared by the DUGKS kernels.
//
// The FP64 helpers keep the operand order of the reference's field
// expressions so the plain FP64 path tracks the CPU oracle to rounding:
//   equilibriumShakhov       discreteVelocity.C:1016-1044
//   equilibriumMaxwellByRho  discreteVelocity.C:1063-1075
//   updateTau                fvDVM.C:808-817
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace dugks {

constexpr double kPi = 3.14159265358979323846;
constexpr double kVSmall = 1.0e-300;

// Everything a step kernel needs besides the distribution buffers.  All
// pointers are device pointers; geometry, DV data and macros are FP64.
struct StepArgs {
    int nC, nI, nW, nA;      // cells, internal faces, wall faces, active faces
    int nV, Vp;              // DVs, padded DV row length
    int D, K, hasH;          // solution directions, KInner, h stored
    double R, Pr, omega, Tref, muRef;
    double dt;
    // geometry
    const double* Sf;        // [nA][3] face area vectors (active faces)
    const double* dO;        // [nA][3] Cf - C_owner
    const double* dN;        // [nI][3] Cf - C_neighbour
    const int* own;          // [nA]
    const int* nei;          // [nI]
    const double* pVec;      // [nI][3] LS vector, owner side
    const double* nVec;      // [nI][3] LS vector, neighbour side
    const double* bVec;      // [nW][3] LS vector of wall faces
    const double* dcW;       // [nW] wall deltaCoeffs
    const double* nHatW;     // [nW][3]
    const double* vol;       // [nC]
    const int* cellOff;      // [nC+1]
    const int* cellFace;     // (activeFace << 1) | side, increasing global face
    // discrete velocities
    const double* xi;        // [3][Vp] (SoA)
    const double* w;         // [Vp] (0 in padding)
    // walls
    const double* Uw;        // [nW][3]
    const double* Tw;        // [nW]
    const double* incAbs;    // [nW] |inComingByRho|
    double* rhoW;            // [nW]
    double* qWall;           // [nW][3]
    double* stressWall;      // [nW][9]
    // macros
    double *rho, *U, *T, *q, *tau;       // cells ([nC], [nC][3], ...)
    double *rhoF, *UF, *TF, *qF, *tauF;  // active faces
    int* status;             // device status word (DUGKS_ERR_NUMERIC on bad state)
    // boundary patches other than diffuse walls (plain FP64 pipeline only);
    // bcMask == 1 << kBcMaxwell when every boundary face is a diffuse wall
    int bcMask;              // bit k set when some boundary face has kind k
    const int* bKind;        // [nW] patch kind of each boundary face (kBc*)
    double* rhoB;            // [nW] rho patch values (pressure patches update them)
    double* TbM;             // [nW] = Tw, writable (pressureOut updates T_b)
    double* UbM;             // [nW][3] = Uw, writable (pressure patches update U_b)
    const double* pB;        // [nW] pressure of the face's pressureIn/Out patch
    const double* bS0;       // [nW][3] area vector of the first face of the face's patch
    const int* symOff;       // [nW] row of symTab for symmetry faces, else -1
    const int* symTab;       // [rows][nV] mirror velocity of each velocity
    // zeroGradient U / T patches (Uvol_/Tvol_.correctBoundaryConditions,
    // fvDVM.C:697-699): bit 0 T, bit 1 U per boundary face; zgMask = their OR
    const int* bZG;          // [nW]
    int zgMask;
};

// Boundary kinds (values of dugks_patch_kind in dugks/dugks.h).
constexpr int kBcEmpty = 0, kBcMaxwell = 1, kBcZeroGradient = 2, kBcFixedValue = 3, kBcFarField = 4,
              kBcPressureIn = 5, kBcPressureOut = 6, kBcSymmetryMod = 7, kBcSymmetryPlane = 8;

#ifdef __CUDACC__
// Index check of the checked build (compiled with -DDUGKS_CHECKED=1, the
// library libdugks_checked.so): an index read from mesh or tile data that is
// outside [0, n) sets the status word to DUGKS_ERR_BOUNDS (8) and is replaced
// by 0, so the access stays inside the array and the step finishes; the host
// reports the error at the next synchronising call.  In the normal build it
// is the index itself.
constexpr int kStatusBounds = 8;
__device__ __forceinline__ int chk(int i, int n, int* status) {
#if defined(DUGKS_CHECKED) && DUGKS_CHECKED
    if ((unsigned)i >= (unsigned)n) {
        atomicExch(status, kStatusBounds);
        return 0;
    }
#else
    (void)n;
    (void)status;
#endif
    return i;
}

__device__ __forceinline__ void shakhov_ref(double rho, double Ux, double Uy, double Uz, double T,
                                            double qx, double qy, double qz, double xx, double xy,
                                            double xz, double R, double Pr, int D, int K, double& gEq,
                                            double& hEq) {
    double ax = Ux - xx, ay = Uy - xy, az = Uz - xz;
    double cSqrByRT = (ax * ax + ay * ay + az * az) / (R * T);
    double cq = ((xx - Ux) * qx + (xy - Uy) * qy + (xz - Uz) * qz) / (5.0 * rho * R * T * R * T);
    double s = sqrt(2.0 * kPi * R * T);
    double pw = (D == 2) ? s * s : (D == 3 ? s * s * s : s);
    double gB = rho / pw * exp(-cSqrByRT / 2.0);
    double pc = (1.0 - Pr) * cq;
    gEq = (1.0 + pc * (cSqrByRT - D - 2.0)) * gB;
    hEq = ((K + 3.0 - D) + pc * ((cSqrByRT - D) * (K + 3.0 - D) - 2 * K)) * gB * R * T;
}

__device__ __forceinline__ double maxwell_by_rho_ref(double Ux, double Uy, double Uz, double T, double xx,
                                                     double xy, double xz, double R, int D) {
    double ax = Ux - xx, ay = Uy - xy, az = Uz - xz;
    double s = sqrt(2.0 * kPi * R * T);
    double pw = (D == 2) ? s * s : (D == 3 ? s * s * s : s);
    return 1.0 / pw * exp(-(ax * ax + ay * ay + az * az) / (2.0 * R * T));
}

__device__ __forceinline__ double tau_ref(double T, double rho, double muRef, double omega, double Tref,
                                          double R) {
    return muRef * exp(omega * log(T / Tref)) / rho / T / R;
}

template <int N>
__device__ __forceinline__ void warp_sum(double (&v)[N]) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
#pragma unroll
        for (int i = 0; i < N; ++i) v[i] += __shfl_xor_sync(0xffffffffu, v[i], o);
}

// Sum N values over the block (blockDim.x multiple of 32, <= 1024).  Every
// thread gets the totals.  smem must hold 32*N doubles.
template <int N>
__device__ __forceinline__ void block_sum(double (&v)[N], double* smem) {
    warp_sum<N>(v);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    __syncthreads();
    if (lane == 0)
#pragma unroll
        for (int i = 0; i < N; ++i) smem[wid * N + i] = v[i];
    __syncthreads();
#pragma unroll
    for (int i = 0; i < N; ++i) v[i] = (lane < nw) ? smem[lane * N + i] : 0.0;
    warp_sum<N>(v);
}

#endif  // __CUDACC__

}  // namespace dugks
