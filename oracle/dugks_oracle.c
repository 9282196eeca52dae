/*
 * dugks_oracle.c -- TEST INFRASTRUCTURE ONLY (parity checker + CPU baseline).
 *
 * FP64 CPU restatement of one DUGKS time step of dugksFoam:
 *   fvDVM::evolution()                  src/fvDVM/fvDVM/fvDVM.C:1086-1108
 * and of the constructor-time set-up it depends on
 *   fvDVM::initialiseDV                 src/fvDVM/fvDVM/fvDVM.C:119-261
 *   fvDVM::setCalculatedMaxwellRhoBC    src/fvDVM/fvDVM/fvDVM.C:263-309
 *   discreteVelocity::initDFtoEq        src/fvDVM/discreteVelocity/discreteVelocity.C:220-249
 *
 * Parity status: UNPINNED.  The reference has no tests or golden outputs and
 * cannot be built here (OpenFOAM + MPI).  Every arithmetic expression below
 * keeps the reference's operand order (OpenFOAM field expressions evaluate
 * left to right, element by element), and every sum keeps the reference's
 * summation order:
 *   - sums over discrete velocities (DVs) run in DV index order, because the
 *     reference accumulates one DV field at a time (forAll(DV_, dvi));
 *   - face-to-cell scatters run in increasing face index, because the
 *     reference loops internal faces then patches in face order.
 * The passes that are independent per DV run DV-parallel (OpenMP); sums run
 * element-parallel with the DV loop sequential, so the result is bit-identical
 * for any thread count.
 *
 * OpenFOAM arithmetic restated here (OpenFOAM >= 2.3, not vendored by the
 * reference; the in-tree restatements are cited):
 *   - least-squares gradient: weights 1/|d|^2 incl. boundary faces,
 *     zeroBoundaryGrad/invDistLeastSquaresVectors.C:100-172; gradient sum as
 *     zeroBoundaryGrad/zeroBoundaryGrad.C:90-133 with the boundary term on;
 *   - boundary delta d_b = n (n.(Cf - C_P)), deltaCoeff_b = 1/|d_b|;
 *   - fixedGradient evaluate: phi_b = phi_P + G_b/deltaCoeff_b;
 *   - inverse of the dd tensor with empty directions padded by 1 and removed;
 *   - primitiveMesh face (triangle fan about the point average) and cell
 *     (pyramids about the face-centre average) centres, areas and volumes.
 * Compile with -ffp-contract=off so x86 and aarch64 give identical bits.
 */
#include "dugks_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define O_VSMALL 1.0e-300
#define O_ROOTVSMALL 1.0e-150
#define O_SMALL 1.0e-15
static const double O_PI = 3.14159265358979323846;

typedef struct oracle_t {
    int nC, nF, nI, nB, nV, D, K, M;
    int* owner;        /* [nF] */
    int* neighbour;    /* [nI] */
    int* bKind;        /* [nB] */
    int* bCell;        /* [nB] */
    double *C, *V;     /* [nC][3], [nC] */
    double *Cf, *Sf;   /* [nF][3] */
    double *pVec, *nVec; /* [nI][3] */
    double* bVec;      /* [nB][3] */
    double* dcI;       /* [nI] */
    double* dcB;       /* [nB] */
    double* nHatB;     /* [nB][3] */
    int *cellOff, *cellFaces; /* active faces per cell, increasing face id */
    double *xi, *w;    /* [nV][3], [nV] */
    double xiMax, R, omega, Tref, muRef, Pr;
    double *Ub, *Tb;   /* [nB][3], [nB]  U, T patch values */
    double *rhob, *pB; /* [nB] rho patch values; pressureIn/Out pressure of the face's patch */
    double* bS0;       /* [nB][3] Sf of the first face of the face's patch (symmetry patches) */
    int* bZG;          /* [nB] bit 0: T patch zeroGradient, bit 1: U patch zeroGradient */
    double *inByRho, *outGoing, *rhoW; /* [nB] */
    double *qWall, *stressWall;        /* [nB][3], [nB][9] */
    double *rho, *U, *T, *q, *tau;     /* cells */
    double *rhoF, *UF, *TF, *qF, *tauF;/* [nF] (empty-patch faces unused) */
    double *gT, *hT;   /* [nV][nC]  g~, h~ */
    double *gB, *hB;   /* [nV][nC]  gBarPvol, hBarPvol internal */
    double *Gg, *Gh;   /* [nV][nB]  fixedGradient gradient of gBarPvol/hBarPvol */
    double *gS, *hS;   /* [nV][nF]  gSurf, hSurf */
    double dt;
} oracle_t;

static void* xcalloc(size_t n, size_t s) {
    void* p = calloc(n ? n : 1, s);
    return p;
}

void oracle_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

/* ---------------------------------------------------------------- vectors */
static inline double dot3(const double* a, const double* b) {
    return a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}
static inline double magsqr3(const double* a) {
    return a[0] * a[0] + a[1] * a[1] + a[2] * a[2];
}

/* --------------------------------------------------------------- geometry */
/* primitiveMesh face centre/area: triangle fan about the point average. */
static void face_geometry(const double* pts, const int* fv, int n, double* Cf, double* Sf) {
    if (n == 3) {
        const double *p0 = pts + 3 * fv[0], *p1 = pts + 3 * fv[1], *p2 = pts + 3 * fv[2];
        double a[3], b[3];
        for (int k = 0; k < 3; ++k) {
            Cf[k] = (1.0 / 3.0) * (p0[k] + p1[k] + p2[k]);
            a[k] = p1[k] - p0[k];
            b[k] = p2[k] - p0[k];
        }
        Sf[0] = 0.5 * (a[1] * b[2] - a[2] * b[1]);
        Sf[1] = 0.5 * (a[2] * b[0] - a[0] * b[2]);
        Sf[2] = 0.5 * (a[0] * b[1] - a[1] * b[0]);
        return;
    }
    double fc[3] = {0, 0, 0};
    for (int i = 0; i < n; ++i)
        for (int k = 0; k < 3; ++k) fc[k] += pts[3 * fv[i] + k];
    for (int k = 0; k < 3; ++k) fc[k] /= n;
    double sumN[3] = {0, 0, 0}, sumA = 0.0, sumAc[3] = {0, 0, 0};
    for (int i = 0; i < n; ++i) {
        const double* p = pts + 3 * fv[i];
        const double* pn = pts + 3 * fv[(i + 1) % n];
        double c[3], a[3], b[3], nv[3];
        for (int k = 0; k < 3; ++k) {
            c[k] = p[k] + pn[k] + fc[k];
            a[k] = pn[k] - p[k];
            b[k] = fc[k] - p[k];
        }
        nv[0] = a[1] * b[2] - a[2] * b[1];
        nv[1] = a[2] * b[0] - a[0] * b[2];
        nv[2] = a[0] * b[1] - a[1] * b[0];
        double am = sqrt(magsqr3(nv));
        for (int k = 0; k < 3; ++k) {
            sumN[k] += nv[k];
            sumAc[k] += am * c[k];
        }
        sumA += am;
    }
    if (sumA < O_ROOTVSMALL) {
        for (int k = 0; k < 3; ++k) { Cf[k] = fc[k]; Sf[k] = 0.0; }
    } else {
        for (int k = 0; k < 3; ++k) {
            Cf[k] = (1.0 / 3.0) * sumAc[k] / sumA;
            Sf[k] = 0.5 * sumN[k];
        }
    }
}

/* 3x3 symmetric inverse by cofactors; t = (xx, xy, xz, yy, yz, zz). */
static void inv_symm(const double* t, double* r) {
    double xx = t[0], xy = t[1], xz = t[2], yy = t[3], yz = t[4], zz = t[5];
    double det = xx * yy * zz + xy * yz * xz + xz * xy * yz - xx * yz * yz - xy * xy * zz - xz * yy * xz;
    r[0] = (yy * zz - yz * yz) / det;
    r[1] = (xz * yz - xy * zz) / det;
    r[2] = (xy * yz - xz * yy) / det;
    r[3] = (xx * zz - xz * xz) / det;
    r[4] = (xy * xz - xx * yz) / det;
    r[5] = (xx * yy - xy * xy) / det;
}

static void symm_dot(const double* t, const double* d, double* r) {
    r[0] = t[0] * d[0] + t[1] * d[1] + t[2] * d[2];
    r[1] = t[1] * d[0] + t[3] * d[1] + t[4] * d[2];
    r[2] = t[2] * d[0] + t[4] * d[1] + t[5] * d[2];
}

/* ---------------------------------------------------------------- physics */
/* discreteVelocity::equilibriumShakhov, discreteVelocity.C:1016-1044 */
static inline void shakhov(const oracle_t* o, double rho, const double* U, double T, const double* q,
                           const double* xi, double* gEq, double* hEq) {
    const double R = o->R, Pr = o->Pr;
    const int D = o->D, K = o->K;
    double umx[3] = {U[0] - xi[0], U[1] - xi[1], U[2] - xi[2]};
    double xmu[3] = {xi[0] - U[0], xi[1] - U[1], xi[2] - U[2]};
    double cSqrByRT = magsqr3(umx) / (R * T);
    double cqBy5pRT = dot3(xmu, q) / (5.0 * rho * R * T * R * T);
    double gEqBGK = rho / pow(sqrt(2.0 * O_PI * R * T), (double)D) * exp(-cSqrByRT / 2.0);
    double pc = (1.0 - Pr) * cqBy5pRT;
    *gEq = (1.0 + pc * (cSqrByRT - D - 2.0)) * gEqBGK;
    *hEq = ((K + 3.0 - D) + pc * ((cSqrByRT - D) * (K + 3.0 - D) - 2 * K)) * gEqBGK * R * T;
}

/* discreteVelocity::equilibriumMaxwellByRho, discreteVelocity.C:1063-1075 */
static inline double maxwell_by_rho(const oracle_t* o, const double* U, double T, const double* xi) {
    double umx[3] = {U[0] - xi[0], U[1] - xi[1], U[2] - xi[2]};
    return 1.0 / pow(sqrt(2.0 * O_PI * o->R * T), (double)o->D) * exp(-magsqr3(umx) / (2.0 * o->R * T));
}

/* discreteVelocity::equilibriumMaxwell for patch fields, discreteVelocity.C:1046-1061 */
static inline void maxwell_patch(const oracle_t* o, double rho, const double* U, double T, const double* xi,
                                 double* geq, double* heq) {
    double umx[3] = {U[0] - xi[0], U[1] - xi[1], U[2] - xi[2]};
    *geq = rho / pow(sqrt(2.0 * O_PI * o->R * T), (double)o->D) * exp(-magsqr3(umx) / (2.0 * o->R * T));
    *heq = (o->K + 3 - o->D) * o->R * T * *geq;
}

/* DV mirrored across a symmetry patch: fvDVM::initialiseDV builds the x, y, z
   mirror ids (fvDVM.C:140-221); the patch picks
   round(|n . (symX, symY, symZ)|) with n its first face's unit normal
   (discreteVelocity.C:733-817). */
static int sym_target(const oracle_t* o, int v, const double* S0) {
    const int M = o->M, D = o->D;
    int ix, iy = 0, iz = 0;
    if (D == 3) { ix = v % M; iy = (v / M) % M; iz = v / (M * M); }
    else if (D == 2) { ix = v % M; iy = v / M; }
    else ix = v;
    double sx, sy, sz;
    if (D == 3) {
        sx = iz * M * M + iy * M + (M - ix - 1);
        sy = iz * M * M + (M - iy - 1) * M + ix;
        sz = (M - iz - 1) * M * M + iy * M + ix;
    } else if (D == 2) {
        sx = iy * M + (M - ix - 1);
        sy = (M - iy - 1) * M + ix;
        sz = 0;
    } else {
        sx = M - ix - 1; sy = 0; sz = 0;
    }
    const double m = sqrt(magsqr3(S0));
    const double n[3] = {S0[0] / m, S0[1] / m, S0[2] / m};
    return (int)round(fabs(n[0] * sx + n[1] * sy + n[2] * sz));
}

/* fvDVM::updateTau, fvDVM.C:808-817 */
static inline double tau_of(const oracle_t* o, double T, double rho) {
    return o->muRef * exp(o->omega * log(T / o->Tref)) / rho / T / o->R;
}

/* -------------------------------------------------------------- set-up */
static void pressure_bc(oracle_t* o);
static void zero_gradient_tu(oracle_t* o);

void* oracle_create(const oracle_case* c) {
    oracle_t* o = (oracle_t*)xcalloc(1, sizeof(oracle_t));
    const int nC = c->nCells, nF = c->nFaces, nI = c->nInternalFaces, nB = nF - nI;
    o->nC = nC; o->nF = nF; o->nI = nI; o->nB = nB;
    o->K = c->KInner;
    o->R = c->R; o->omega = c->omega; o->Tref = c->Tref; o->muRef = c->muRef; o->Pr = c->Pr;
    o->xiMax = c->xiMax;
    o->owner = (int*)xcalloc(nF, sizeof(int));
    o->neighbour = (int*)xcalloc(nI, sizeof(int));
    memcpy(o->owner, c->owner, sizeof(int) * nF);
    memcpy(o->neighbour, c->neighbour, sizeof(int) * nI);
    o->bKind = (int*)xcalloc(nB, sizeof(int));
    o->bCell = (int*)xcalloc(nB, sizeof(int));
    for (int p = 0; p < c->nPatches; ++p)
        for (int i = 0; i < c->patchSize[p]; ++i) o->bKind[c->patchStart[p] + i - nI] = c->patchKind[p];
    for (int b = 0; b < nB; ++b) o->bCell[b] = c->owner[nI + b];

    /* primitiveMesh geometry over ALL faces (empty ones included). */
    o->Cf = (double*)xcalloc(3 * (size_t)nF, sizeof(double));
    o->Sf = (double*)xcalloc(3 * (size_t)nF, sizeof(double));
    for (int f = 0; f < nF; ++f)
        face_geometry(c->points, c->faceVerts + c->faceOffsets[f], c->faceOffsets[f + 1] - c->faceOffsets[f],
                      o->Cf + 3 * f, o->Sf + 3 * f);
    double* cEst = (double*)xcalloc(3 * (size_t)nC, sizeof(double));
    int* nCF = (int*)xcalloc(nC, sizeof(int));
    for (int f = 0; f < nF; ++f) {
        int ow = c->owner[f];
        for (int k = 0; k < 3; ++k) cEst[3 * ow + k] += o->Cf[3 * f + k];
        nCF[ow]++;
    }
    for (int f = 0; f < nI; ++f) {
        int ne = c->neighbour[f];
        for (int k = 0; k < 3; ++k) cEst[3 * ne + k] += o->Cf[3 * f + k];
        nCF[ne]++;
    }
    for (int i = 0; i < nC; ++i)
        for (int k = 0; k < 3; ++k) cEst[3 * i + k] /= nCF[i];
    o->C = (double*)xcalloc(3 * (size_t)nC, sizeof(double));
    o->V = (double*)xcalloc(nC, sizeof(double));
    for (int f = 0; f < nF; ++f) {
        int ow = c->owner[f];
        double d[3], pc[3];
        for (int k = 0; k < 3; ++k) d[k] = o->Cf[3 * f + k] - cEst[3 * ow + k];
        double pyr3 = dot3(o->Sf + 3 * f, d);
        for (int k = 0; k < 3; ++k) pc[k] = (3.0 / 4.0) * o->Cf[3 * f + k] + (1.0 / 4.0) * cEst[3 * ow + k];
        for (int k = 0; k < 3; ++k) o->C[3 * ow + k] += pyr3 * pc[k];
        o->V[ow] += pyr3;
    }
    for (int f = 0; f < nI; ++f) {
        int ne = c->neighbour[f];
        double d[3], pc[3];
        for (int k = 0; k < 3; ++k) d[k] = cEst[3 * ne + k] - o->Cf[3 * f + k];
        double pyr3 = dot3(o->Sf + 3 * f, d);
        for (int k = 0; k < 3; ++k) pc[k] = (3.0 / 4.0) * o->Cf[3 * f + k] + (1.0 / 4.0) * cEst[3 * ne + k];
        for (int k = 0; k < 3; ++k) o->C[3 * ne + k] += pyr3 * pc[k];
        o->V[ne] += pyr3;
    }
    for (int i = 0; i < nC; ++i) {
        for (int k = 0; k < 3; ++k) o->C[3 * i + k] /= o->V[i];
        o->V[i] *= (1.0 / 3.0);
    }
    free(cEst);
    free(nCF);

    /* Solution directions: a direction is empty when the empty patches'
       face normals point along it (2D front/back -> z removed). */
    double emptyDir[3] = {0, 0, 0};
    int nEmpty = 0;
    for (int b = 0; b < nB; ++b)
        if (o->bKind[b] == ORACLE_PATCH_EMPTY) {
            const double* s = o->Sf + 3 * (nI + b);
            double m = sqrt(magsqr3(s));
            for (int k = 0; k < 3; ++k) emptyDir[k] += fabs(s[k]) / m;
            nEmpty++;
        }
    int D = 3;
    int isEmpty[3] = {0, 0, 0};
    if (nEmpty > 0) {
        double m = sqrt(magsqr3(emptyDir));
        for (int k = 0; k < 3; ++k)
            if (emptyDir[k] / m > 1e-6) { isEmpty[k] = 1; D--; }
    }
    o->D = D;

    /* deltaCoeffs, boundary deltas */
    o->dcI = (double*)xcalloc(nI, sizeof(double));
    o->dcB = (double*)xcalloc(nB, sizeof(double));
    o->nHatB = (double*)xcalloc(3 * (size_t)nB, sizeof(double));
    double* dB = (double*)xcalloc(3 * (size_t)nB, sizeof(double));
    for (int f = 0; f < nI; ++f) {
        double d[3];
        for (int k = 0; k < 3; ++k) d[k] = o->C[3 * c->neighbour[f] + k] - o->C[3 * c->owner[f] + k];
        o->dcI[f] = 1.0 / sqrt(magsqr3(d));
    }
    for (int b = 0; b < nB; ++b) {
        if (o->bKind[b] == ORACLE_PATCH_EMPTY) continue;
        int f = nI + b, P = o->bCell[b];
        double magSf = sqrt(magsqr3(o->Sf + 3 * f));
        double n[3], r[3];
        for (int k = 0; k < 3; ++k) {
            n[k] = o->Sf[3 * f + k] / magSf;
            r[k] = o->Cf[3 * f + k] - o->C[3 * P + k];
        }
        double s = dot3(n, r);
        for (int k = 0; k < 3; ++k) {
            o->nHatB[3 * b + k] = n[k];
            dB[3 * b + k] = n[k] * s;
        }
        o->dcB[b] = 1.0 / sqrt(magsqr3(dB + 3 * b));
    }

    /* least-squares vectors, invDistLeastSquaresVectors.C:100-172 */
    double* dd = (double*)xcalloc(6 * (size_t)nC, sizeof(double));
    for (int f = 0; f < nI; ++f) {
        int ow = c->owner[f], ne = c->neighbour[f];
        double d[3];
        for (int k = 0; k < 3; ++k) d[k] = o->C[3 * ne + k] - o->C[3 * ow + k];
        double m2 = magsqr3(d);
        double wdd[6] = {d[0] * d[0] / m2, d[0] * d[1] / m2, d[0] * d[2] / m2,
                         d[1] * d[1] / m2, d[1] * d[2] / m2, d[2] * d[2] / m2};
        for (int k = 0; k < 6; ++k) { dd[6 * ow + k] += wdd[k]; dd[6 * ne + k] += wdd[k]; }
    }
    for (int b = 0; b < nB; ++b) {
        if (o->bKind[b] == ORACLE_PATCH_EMPTY) continue;
        int P = o->bCell[b];
        const double* d = dB + 3 * b;
        double m2 = magsqr3(d);
        double wdd[6] = {d[0] * d[0] / m2, d[0] * d[1] / m2, d[0] * d[2] / m2,
                         d[1] * d[1] / m2, d[1] * d[2] / m2, d[2] * d[2] / m2};
        for (int k = 0; k < 6; ++k) dd[6 * P + k] += wdd[k];
    }
    double* invDd = (double*)xcalloc(6 * (size_t)nC, sizeof(double));
    const int diag[3] = {0, 3, 5};
    for (int i = 0; i < nC; ++i) {
        double t[6];
        memcpy(t, dd + 6 * i, sizeof(t));
        for (int k = 0; k < 3; ++k) if (isEmpty[k]) t[diag[k]] += 1.0;
        inv_symm(t, invDd + 6 * i);
        for (int k = 0; k < 3; ++k) if (isEmpty[k]) invDd[6 * i + diag[k]] -= 1.0;
    }
    o->pVec = (double*)xcalloc(3 * (size_t)nI, sizeof(double));
    o->nVec = (double*)xcalloc(3 * (size_t)nI, sizeof(double));
    o->bVec = (double*)xcalloc(3 * (size_t)nB, sizeof(double));
    for (int f = 0; f < nI; ++f) {
        int ow = c->owner[f], ne = c->neighbour[f];
        double d[3], a[3], b2[3];
        for (int k = 0; k < 3; ++k) d[k] = o->C[3 * ne + k] - o->C[3 * ow + k];
        double m2 = magsqr3(d);
        symm_dot(invDd + 6 * ow, d, a);
        symm_dot(invDd + 6 * ne, d, b2);
        for (int k = 0; k < 3; ++k) {
            o->pVec[3 * f + k] = a[k] / m2;
            o->nVec[3 * f + k] = -(b2[k] / m2);
        }
    }
    for (int b = 0; b < nB; ++b) {
        if (o->bKind[b] == ORACLE_PATCH_EMPTY) continue;
        const double* d = dB + 3 * b;
        double m2 = magsqr3(d), a[3];
        symm_dot(invDd + 6 * o->bCell[b], d, a);
        for (int k = 0; k < 3; ++k) o->bVec[3 * b + k] = a[k] / m2;
    }
    free(dd);
    free(invDd);
    free(dB);

    /* cell -> active face lists, increasing face index */
    o->cellOff = (int*)xcalloc(nC + 1, sizeof(int));
    for (int f = 0; f < nF; ++f) {
        if (f >= nI && o->bKind[f - nI] == ORACLE_PATCH_EMPTY) continue;
        o->cellOff[c->owner[f] + 1]++;
        if (f < nI) o->cellOff[c->neighbour[f] + 1]++;
    }
    for (int i = 0; i < nC; ++i) o->cellOff[i + 1] += o->cellOff[i];
    o->cellFaces = (int*)xcalloc(o->cellOff[nC], sizeof(int));
    int* fill = (int*)xcalloc(nC, sizeof(int));
    for (int f = 0; f < nF; ++f) {
        if (f >= nI && o->bKind[f - nI] == ORACLE_PATCH_EMPTY) continue;
        int ow = c->owner[f];
        o->cellFaces[o->cellOff[ow] + fill[ow]++] = f;
        if (f < nI) {
            int ne = c->neighbour[f];
            o->cellFaces[o->cellOff[ne] + fill[ne]++] = f;
        }
    }
    free(fill);

    /* DV set, fvDVM::initialiseDV fvDVM.C:140-221 */
    const int M = c->nXiPerDim;
    int nV = (D == 3) ? M * M * M : (D == 2 ? M * M : M);
    o->nV = nV;
    o->M = M;
    o->xi = (double*)xcalloc(3 * (size_t)nV, sizeof(double));
    o->w = (double*)xcalloc(nV, sizeof(double));
    {
        int i = 0;
        if (D == 3) {
            for (int iz = 0; iz < M; ++iz)
                for (int iy = 0; iy < M; ++iy)
                    for (int ix = 0; ix < M; ++ix, ++i) {
                        o->w[i] = c->weights[iz] * c->weights[iy] * c->weights[ix];
                        o->xi[3 * i] = c->xis[ix]; o->xi[3 * i + 1] = c->xis[iy]; o->xi[3 * i + 2] = c->xis[iz];
                    }
        } else if (D == 2) {
            for (int iy = 0; iy < M; ++iy)
                for (int ix = 0; ix < M; ++ix, ++i) {
                    o->w[i] = c->weights[iy] * c->weights[ix] * 1;
                    o->xi[3 * i] = c->xis[ix]; o->xi[3 * i + 1] = c->xis[iy]; o->xi[3 * i + 2] = 0.0;
                }
        } else {
            for (int ix = 0; ix < M; ++ix, ++i) {
                o->w[i] = c->weights[ix] * 1 * 1;
                o->xi[3 * i] = c->xis[ix];
            }
        }
    }

    /* wall data */
    o->Ub = (double*)xcalloc(3 * (size_t)nB, sizeof(double));
    o->Tb = (double*)xcalloc(nB, sizeof(double));
    memcpy(o->Ub, c->Ub, sizeof(double) * 3 * nB);
    memcpy(o->Tb, c->Tb, sizeof(double) * nB);
    o->rhob = (double*)xcalloc(nB, sizeof(double));
    o->pB = (double*)xcalloc(nB, sizeof(double));
    o->bS0 = (double*)xcalloc(3 * (size_t)nB, sizeof(double));
    o->bZG = (int*)xcalloc(nB, sizeof(int));
    if (c->rhob) memcpy(o->rhob, c->rhob, sizeof(double) * nB);
    for (int p = 0; p < c->nPatches; ++p) {
        for (int i = 0; i < c->patchSize[p]; ++i) {
            const int b = c->patchStart[p] + i - nI;
            if (c->patchPressure) o->pB[b] = c->patchPressure[p];
            o->bZG[b] = (c->patchTzg && c->patchTzg[p] ? 1 : 0) | (c->patchUzg && c->patchUzg[p] ? 2 : 0);
            for (int d = 0; d < 3; ++d) o->bS0[3 * b + d] = o->Sf[3 * (size_t)c->patchStart[p] + d];
        }
    }
    o->inByRho = (double*)xcalloc(nB, sizeof(double));
    o->outGoing = (double*)xcalloc(nB, sizeof(double));
    o->rhoW = (double*)xcalloc(nB, sizeof(double));
    o->qWall = (double*)xcalloc(3 * (size_t)nB, sizeof(double));
    o->stressWall = (double*)xcalloc(9 * (size_t)nB, sizeof(double));
    for (int b = 0; b < nB; ++b) o->rhoW[b] = 1.0; /* calculatedMaxwell ctor value */

    /* macros */
    o->rho = (double*)xcalloc(nC, sizeof(double));
    o->U = (double*)xcalloc(3 * (size_t)nC, sizeof(double));
    o->T = (double*)xcalloc(nC, sizeof(double));
    o->q = (double*)xcalloc(3 * (size_t)nC, sizeof(double));
    o->tau = (double*)xcalloc(nC, sizeof(double));
    memcpy(o->rho, c->rho0, sizeof(double) * nC);
    memcpy(o->U, c->U0, sizeof(double) * 3 * nC);
    memcpy(o->T, c->T0, sizeof(double) * nC);
    o->rhoF = (double*)xcalloc(nF, sizeof(double));
    o->UF = (double*)xcalloc(3 * (size_t)nF, sizeof(double));
    o->TF = (double*)xcalloc(nF, sizeof(double));
    o->qF = (double*)xcalloc(3 * (size_t)nF, sizeof(double));
    o->tauF = (double*)xcalloc(nF, sizeof(double));

    size_t nVC = (size_t)nV * nC, nVF = (size_t)nV * nF, nVB = (size_t)nV * nB;
    o->gT = (double*)xcalloc(nVC, sizeof(double));
    o->hT = (double*)xcalloc(nVC, sizeof(double));
    o->gB = (double*)xcalloc(nVC, sizeof(double));
    o->hB = (double*)xcalloc(nVC, sizeof(double));
    o->Gg = (double*)xcalloc(nVB, sizeof(double));
    o->Gh = (double*)xcalloc(nVB, sizeof(double));
    o->gS = (double*)xcalloc(nVF, sizeof(double));
    o->hS = (double*)xcalloc(nVF, sizeof(double));

    /* discreteVelocity::initDFtoEq (q = 0), discreteVelocity.C:220-249 */
    const double q0[3] = {0, 0, 0};
#pragma omp parallel for schedule(dynamic, 4)
    for (int v = 0; v < nV; ++v)
        for (int i = 0; i < nC; ++i)
            shakhov(o, o->rho[i], o->U + 3 * i, o->T[i], q0, o->xi + 3 * v,
                    o->gT + (size_t)v * nC + i, o->hT + (size_t)v * nC + i);

    /* a zeroGradient U or T patch, as constructed from its field file, holds
       the owner cells' initial values */
    zero_gradient_tu(o);
    /* discreteVelocity::initBoundaryField (discreteVelocity.C:302-345): the
       mixed patches (rho fixedValue) start at the Maxwellian of the patch values;
       their incoming DFs are never written again. */
    for (int b = 0; b < nB; ++b) {
        if (o->bKind[b] != ORACLE_PATCH_FIXED_VALUE) continue;
        const int f = nI + b;
        for (int v = 0; v < nV; ++v)
            maxwell_patch(o, o->rhob[b], o->Ub + 3 * b, o->Tb[b], o->xi + 3 * v, o->gS + (size_t)v * nF + f,
                          o->hS + (size_t)v * nF + f);
    }

    /* fvDVM::setCalculatedMaxwellRhoBC, fvDVM.C:263-309 (computed once) */
    for (int b = 0; b < nB; ++b) {
        if (o->bKind[b] != ORACLE_PATCH_MAXWELL) continue;
        const double* S = o->Sf + 3 * (nI + b);
        double acc = 0.0;
        for (int v = 0; v < nV; ++v) {
            double xs = dot3(o->xi + 3 * v, S);
            if (xs < 0) acc += -o->w[v] * xs * maxwell_by_rho(o, o->Ub + 3 * b, o->Tb[b], o->xi + 3 * v);
        }
        o->inByRho[b] = acc;
    }
    /* tauVol at construction; Usurf = linear interpolate(U) for the first CFL */
    for (int i = 0; i < nC; ++i) o->tau[i] = tau_of(o, o->T[i], o->rho[i]);
    for (int f = 0; f < nI; ++f) {
        int ow = c->owner[f], ne = c->neighbour[f];
        double a[3], bb[3];
        for (int k = 0; k < 3; ++k) {
            a[k] = o->Cf[3 * f + k] - o->C[3 * ow + k];
            bb[k] = o->C[3 * ne + k] - o->Cf[3 * f + k];
        }
        double sO = fabs(dot3(o->Sf + 3 * f, a)), sN = fabs(dot3(o->Sf + 3 * f, bb));
        double wl = sN / (sO + sN);
        for (int k = 0; k < 3; ++k) o->UF[3 * f + k] = wl * o->U[3 * ow + k] + (1.0 - wl) * o->U[3 * ne + k];
    }
    for (int b = 0; b < nB; ++b)
        for (int k = 0; k < 3; ++k) o->UF[3 * (nI + b) + k] = o->Ub[3 * b + k];
    /* the constructor ends with updatePressureInOutBC on the initial macros
       (fvDVM.C:1067-1071: "set initial rho in pressureIn/Out BC") */
    pressure_bc(o);
    return o;
}

void oracle_destroy(void* h) {
    oracle_t* o = (oracle_t*)h;
    if (!o) return;
    void* ptrs[] = {o->owner, o->neighbour, o->bKind, o->bCell, o->C, o->V, o->Cf, o->Sf, o->pVec, o->nVec,
                    o->bVec, o->dcI, o->dcB, o->nHatB, o->cellOff, o->cellFaces, o->xi, o->w, o->Ub, o->Tb,
                    o->inByRho, o->outGoing, o->rhoW, o->qWall, o->stressWall, o->rho, o->U, o->T, o->q,
                    o->rhob, o->pB, o->bS0, o->bZG,
                    o->tau, o->rhoF, o->UF, o->TF, o->qF, o->tauF, o->gT, o->hT, o->gB, o->hB, o->Gg, o->Gh,
                    o->gS, o->hS};
    for (size_t i = 0; i < sizeof(ptrs) / sizeof(ptrs[0]); ++i) free(ptrs[i]);
    free(o);
}

int oracle_nsolutiond(void* h) { return ((oracle_t*)h)->D; }
int oracle_ndv(void* h) { return ((oracle_t*)h)->nV; }

/* ---------------------------------------------------------------- passes */
/* P1 discreteVelocity::updateGHbarPvol (discreteVelocity.C:346-410) for DV v,
   then P2/P3 discreteVelocity::updateGHbarSurf (discreteVelocity.C:412-691):
   least-squares gradient, lagged fixedGradient update, face reconstruction. */
static void dv_bar_and_surf(oracle_t* o, int v, double* grad /* [nC][3] */, double* grh) {
    const int nC = o->nC, nI = o->nI, nB = o->nB, nF = o->nF;
    const double dt = o->dt;
    const double* xi = o->xi + 3 * v;
    double* gT = o->gT + (size_t)v * nC;
    double* hT = o->hT + (size_t)v * nC;
    double* gB = o->gB + (size_t)v * nC;
    double* hB = o->hB + (size_t)v * nC;
    double* Gg = o->Gg + (size_t)v * nB;
    double* Gh = o->Gh + (size_t)v * nB;
    double* gS = o->gS + (size_t)v * nF;
    double* hS = o->hS + (size_t)v * nF;

    /* P1: relax toward Shakhov; relaxFactor = 1.5 dt/(2 tau + dt) */
    for (int i = 0; i < nC; ++i) {
        double a = 1.5 * dt / (2.0 * o->tau[i] + dt);
        double ge, he;
        shakhov(o, o->rho[i], o->U + 3 * i, o->T[i], o->q + 3 * i, xi, &ge, &he);
        gB[i] = (1.0 - a) * gT[i] + a * ge;
        hB[i] = (1.0 - a) * hT[i] + a * he;
    }
    /* P2: leastSquares grad of gBarPvol with fixedGradient boundary values */
    for (int i = 0; i < nC; ++i) {
        double gg[3] = {0, 0, 0}, hg[3] = {0, 0, 0};
        for (int j = o->cellOff[i]; j < o->cellOff[i + 1]; ++j) {
            int f = o->cellFaces[j];
            if (f < nI) {
                int ow = o->owner[f], ne = o->neighbour[f];
                double dg = gB[ne] - gB[ow], dh = hB[ne] - hB[ow];
                if (i == ow) {
                    for (int k = 0; k < 3; ++k) { gg[k] += o->pVec[3 * f + k] * dg; hg[k] += o->pVec[3 * f + k] * dh; }
                } else {
                    for (int k = 0; k < 3; ++k) { gg[k] -= o->nVec[3 * f + k] * dg; hg[k] -= o->nVec[3 * f + k] * dh; }
                }
            } else {
                int b = f - nI;
                double gbv, hbv;
                if (o->bKind[b] == ORACLE_PATCH_SYMMETRY_PLANE) {
                    /* constraint patch of gBarPvol: scalar symmetryPlane value = internal value */
                    gbv = gB[i];
                    hbv = hB[i];
                } else {
                    gbv = gB[i] + Gg[b] / o->dcB[b];  /* fixedGradient evaluate */
                    hbv = hB[i] + Gh[b] / o->dcB[b];
                }
                double dg = gbv - gB[i], dh = hbv - hB[i];
                for (int k = 0; k < 3; ++k) { gg[k] += o->bVec[3 * b + k] * dg; hg[k] += o->bVec[3 * b + k] * dh; }
            }
        }
        for (int k = 0; k < 3; ++k) { grad[3 * i + k] = gg[k]; grh[3 * i + k] = hg[k]; }
    }
    /* lagged boundary gradient for the next step: G_b = (grad_P).n */
    for (int b = 0; b < nB; ++b) {
        if (o->bKind[b] == ORACLE_PATCH_EMPTY) continue;
        int P = o->bCell[b];
        Gg[b] = dot3(grad + 3 * P, o->nHatB + 3 * b);
        Gh[b] = dot3(grh + 3 * P, o->nHatB + 3 * b);
    }
    /* P3: internal faces, upwind linear reconstruction with the -xi dt/2 shift */
    for (int f = 0; f < nI; ++f) {
        int ow = o->owner[f], ne = o->neighbour[f];
        double xs = dot3(xi, o->Sf + 3 * f);
        double rO[3], rN[3];
        for (int k = 0; k < 3; ++k) {
            rO[k] = o->Cf[3 * f + k] - o->C[3 * ow + k] - 0.5 * xi[k] * dt;
            rN[k] = o->Cf[3 * f + k] - o->C[3 * ne + k] - 0.5 * xi[k] * dt;
        }
        if (xs >= O_VSMALL) {
            gS[f] = gB[ow] + dot3(grad + 3 * ow, rO);
            hS[f] = hB[ow] + dot3(grh + 3 * ow, rO);
        } else if (xs < -O_VSMALL) {
            gS[f] = gB[ne] + dot3(grad + 3 * ne, rN);
            hS[f] = hB[ne] + dot3(grh + 3 * ne, rN);
        } else {
            gS[f] = 0.5 * (gB[ne] + dot3(grad + 3 * ne, rN) + gB[ow] + dot3(grad + 3 * ow, rO));
            hS[f] = 0.5 * (hB[ne] + dot3(grh + 3 * ne, rN) + hB[ow] + dot3(grh + 3 * ow, rO));
        }
    }
    /* P3: boundary faces by surface patch type (discreteVelocity.C:530-689) */
    for (int b = 0; b < nB; ++b) {
        const int kind = o->bKind[b];
        if (kind == ORACLE_PATCH_EMPTY) continue;
        int f = nI + b, P = o->bCell[b];
        const double xs = dot3(xi, o->Sf + 3 * f);
        int outgoing;
        if (kind == ORACLE_PATCH_ZERO_GRADIENT) {
            /* gSurf == gBarPvol patchInternalField, every DV */
            gS[f] = gB[P];
            hS[f] = hB[P];
            continue;
        } else if (kind == ORACLE_PATCH_SYMMETRY_MOD || kind == ORACLE_PATCH_SYMMETRY_PLANE) {
            outgoing = xs > -O_VSMALL;  /* outgoing and tangential */
        } else {
            outgoing = xs > 0;
        }
        if (outgoing) {
            double r[3];
            for (int k = 0; k < 3; ++k) r[k] = o->Cf[3 * f + k] - o->C[3 * P + k] - 0.5 * xi[k] * dt;
            gS[f] = gB[P] + dot3(grad + 3 * P, r);
            hS[f] = hB[P] + dot3(grh + 3 * P, r);
        } else if (kind == ORACLE_PATCH_FAR_FIELD || kind == ORACLE_PATCH_PRESSURE_IN ||
                   kind == ORACLE_PATCH_PRESSURE_OUT) {
            /* incoming: rho_b M(U of the owner cell, T_b) */
            gS[f] = o->rhob[b] * maxwell_by_rho(o, o->U + 3 * P, o->Tb[b], xi);
            hS[f] = gS[f] * (o->R * o->Tb[b]) * (o->K + 3 - o->D);
        }
    }
}

/* P5 discreteVelocity::updateGHbarSurfMaxwellWallIn (discreteVelocity.C:693-731) */
static void dv_wall_in(oracle_t* o, int v) {
    const int nI = o->nI, nB = o->nB, nF = o->nF;
    const double* xi = o->xi + 3 * v;
    double* gS = o->gS + (size_t)v * nF;
    double* hS = o->hS + (size_t)v * nF;
    for (int b = 0; b < nB; ++b) {
        if (o->bKind[b] != ORACLE_PATCH_MAXWELL) continue;
        int f = nI + b;
        if (dot3(xi, o->Sf + 3 * f) <= 0) {
            gS[f] = o->rhoW[b] * maxwell_by_rho(o, o->Ub + 3 * b, o->Tb[b], xi);
            hS[f] = gS[f] * (o->R * o->Tb[b]) * (o->K + 3 - o->D);
        }
    }
}

/* P7 discreteVelocity::updateGHsurf (discreteVelocity.C:819-932), then
   P8 discreteVelocity::updateGHtildeVol (discreteVelocity.C:934-978). */
static void dv_surf_and_tilde(oracle_t* o, int v) {
    const int nC = o->nC, nI = o->nI, nB = o->nB, nF = o->nF;
    const double dt = o->dt, hh = 0.5 * dt;
    const double* xi = o->xi + 3 * v;
    double* gS = o->gS + (size_t)v * nF;
    double* hS = o->hS + (size_t)v * nF;
    double* gT = o->gT + (size_t)v * nC;
    double* hT = o->hT + (size_t)v * nC;
    const double* gB = o->gB + (size_t)v * nC;
    const double* hB = o->hB + (size_t)v * nC;
    for (int f = 0; f < nI; ++f) {
        double b = hh / (2 * o->tauF[f] + hh);
        double ge, he;
        shakhov(o, o->rhoF[f], o->UF + 3 * f, o->TF[f], o->qF + 3 * f, xi, &ge, &he);
        gS[f] = (1.0 - b) * gS[f] + b * ge;
        hS[f] = (1.0 - b) * hS[f] + b * he;
    }
    /* Boundary patches.  The field assignment is a no-op on the project's own
       surface patch types (maxwellWall, mixed, farField, zeroGradient,
       DVMsymmetry: e.g. maxwellWallFvsPatchField.H:163-181) and a plain
       assignment on the constraint type symmetryPlane; then every outgoing DV
       (xi.S > 0) is relaxed explicitly (discreteVelocity.C:887-931), so
       symmetryPlane relaxes its outgoing DVs twice. */
    for (int bb = 0; bb < nB; ++bb) {
        const int kind = o->bKind[bb];
        if (kind == ORACLE_PATCH_EMPTY) continue;
        int f = nI + bb;
        const int out = dot3(xi, o->Sf + 3 * f) > 0;
        const int times = (kind == ORACLE_PATCH_SYMMETRY_PLANE) + out;
        if (times == 0) continue;
        double b = hh / (2 * o->tauF[f] + hh);
        double ge, he;
        shakhov(o, o->rhoF[f], o->UF + 3 * f, o->TF[f], o->qF + 3 * f, xi, &ge, &he);
        for (int t = 0; t < times; ++t) {
            gS[f] = (1.0 - b) * gS[f] + b * ge;
            hS[f] = (1.0 - b) * hS[f] + b * he;
        }
    }
    /* P8 */
    for (int i = 0; i < nC; ++i) {
        double g = -1.0 / 3 * gT[i] + 4.0 / 3 * gB[i];
        double h = -1.0 / 3 * hT[i] + 4.0 / 3 * hB[i];
        for (int j = o->cellOff[i]; j < o->cellOff[i + 1]; ++j) {
            int f = o->cellFaces[j];
            double xs = dot3(xi, o->Sf + 3 * f);
            if (f < nI && o->neighbour[f] == i) {
                g += xs * gS[f] * dt / o->V[i];
                h += xs * hS[f] * dt / o->V[i];
            } else {
                g -= xs * gS[f] * dt / o->V[i];
                h -= xs * hS[f] * dt / o->V[i];
            }
        }
        gT[i] = g;
        hT[i] = h;
    }
}

#define O_BLK 64

/* P6 fvDVM::updateMacroSurf (fvDVM.C:456-582): face moments in DV order. */
static void face_macros(oracle_t* o) {
    const int nF = o->nF, nI = o->nI, nV = o->nV;
    const double dt = o->dt;
    const double c1 = (o->K + 3) / 2.0 * o->R;
#pragma omp parallel for schedule(dynamic, 1)
    for (int f0 = 0; f0 < nF; f0 += O_BLK) {
        int f1 = f0 + O_BLK < nF ? f0 + O_BLK : nF;
        double rho[O_BLK], ru[O_BLK][3], re[O_BLK], qq[O_BLK][3];
        for (int f = f0; f < f1; ++f) {
            rho[f - f0] = 0; re[f - f0] = 0;
            for (int k = 0; k < 3; ++k) { ru[f - f0][k] = 0; qq[f - f0][k] = 0; }
        }
        for (int v = 0; v < nV; ++v) {
            const double* xi = o->xi + 3 * v;
            const double w = o->w[v];
            const double xi2 = magsqr3(xi);
            const double* gS = o->gS + (size_t)v * nF;
            const double* hS = o->hS + (size_t)v * nF;
            for (int f = f0; f < f1; ++f) {
                if (f >= nI && o->bKind[f - nI] == ORACLE_PATCH_EMPTY) continue;
                int l = f - f0;
                rho[l] += w * gS[f];
                for (int k = 0; k < 3; ++k) ru[l][k] += w * gS[f] * xi[k];
                re[l] += 0.5 * w * (gS[f] * xi2 + hS[f]);
            }
        }
        for (int f = f0; f < f1; ++f) {
            if (f >= nI && o->bKind[f - nI] == ORACLE_PATCH_EMPTY) continue;
            int l = f - f0;
            o->rhoF[f] = rho[l];
            for (int k = 0; k < 3; ++k) o->UF[3 * f + k] = ru[l][k] / rho[l];
            o->TF[f] = (re[l] - 0.5 * rho[l] * magsqr3(o->UF + 3 * f)) / (c1 * rho[l]);
            o->tauF[f] = tau_of(o, o->TF[f], o->rhoF[f]);
        }
        for (int v = 0; v < nV; ++v) {
            const double* xi = o->xi + 3 * v;
            const double w = o->w[v];
            const double* gS = o->gS + (size_t)v * nF;
            const double* hS = o->hS + (size_t)v * nF;
            for (int f = f0; f < f1; ++f) {
                if (f >= nI && o->bKind[f - nI] == ORACLE_PATCH_EMPTY) continue;
                int l = f - f0;
                double c[3] = {xi[0] - o->UF[3 * f], xi[1] - o->UF[3 * f + 1], xi[2] - o->UF[3 * f + 2]};
                double s = magsqr3(c) * gS[f] + hS[f];
                for (int k = 0; k < 3; ++k) qq[l][k] += 0.5 * w * c[k] * s;
            }
        }
        for (int f = f0; f < f1; ++f) {
            if (f >= nI && o->bKind[f - nI] == ORACLE_PATCH_EMPTY) continue;
            int l = f - f0;
            double fac = 2.0 * o->tauF[f] / (2.0 * o->tauF[f] + 0.5 * dt * o->Pr);
            for (int k = 0; k < 3; ++k) o->qF[3 * f + k] = fac * qq[l][k];
        }
    }
    /* wall heat flux and stress (fvDVM.C:539-581), face-outer, DV-inner */
    const int nB = o->nB;
#pragma omp parallel for schedule(dynamic, 4)
    for (int b = 0; b < nB; ++b) {
        double* qw = o->qWall + 3 * b;
        double* sw = o->stressWall + 9 * b;
        for (int k = 0; k < 3; ++k) qw[k] = 0.0;
        for (int k = 0; k < 9; ++k) sw[k] = 0.0;
        if (o->bKind[b] != ORACLE_PATCH_MAXWELL) continue;
        int f = nI + b;
        for (int v = 0; v < nV; ++v) {
            const double* xi = o->xi + 3 * v;
            double w = o->w[v];
            double g = o->gS[(size_t)v * nF + f], h = o->hS[(size_t)v * nF + f];
            double c[3] = {xi[0] - o->Ub[3 * b], xi[1] - o->Ub[3 * b + 1], xi[2] - o->Ub[3 * b + 2]};
            double s = magsqr3(c) * g + h;
            for (int k = 0; k < 3; ++k) qw[k] += 0.5 * 1.0 * w * c[k] * s;
            double wg = 1.0 * w * g;
            for (int r = 0; r < 3; ++r)
                for (int k = 0; k < 3; ++k) sw[3 * r + k] += wg * xi[r] * xi[k];
        }
        double tw = o->tauF[f];
        double fq = 2.0 * tw / (2.0 * tw + 0.5 * dt * o->Pr);
        double fs = 2.0 * tw / (2.0 * tw + 0.5 * dt);
        for (int k = 0; k < 3; ++k) qw[k] = fq * qw[k];
        for (int k = 0; k < 9; ++k) sw[k] = fs * sw[k];
    }
}

/* P9 fvDVM::updateMacroVol (fvDVM.C:597-728), macroFlux "no" branch */
static void cell_macros(oracle_t* o) {
    const int nC = o->nC, nV = o->nV;
    const double dt = o->dt;
    const double c1 = (o->K + 3) / 2.0 * o->R;
#pragma omp parallel for schedule(dynamic, 1)
    for (int i0 = 0; i0 < nC; i0 += O_BLK) {
        int i1 = i0 + O_BLK < nC ? i0 + O_BLK : nC;
        double rho[O_BLK], ru[O_BLK][3], re[O_BLK], qq[O_BLK][3];
        for (int i = i0; i < i1; ++i) {
            rho[i - i0] = 0; re[i - i0] = 0;
            for (int k = 0; k < 3; ++k) { ru[i - i0][k] = 0; qq[i - i0][k] = 0; }
        }
        for (int v = 0; v < nV; ++v) {
            const double* xi = o->xi + 3 * v;
            const double w = o->w[v];
            const double xi2 = magsqr3(xi);
            const double* gT = o->gT + (size_t)v * nC;
            const double* hT = o->hT + (size_t)v * nC;
            for (int i = i0; i < i1; ++i) {
                int l = i - i0;
                rho[l] += w * gT[i];
                for (int k = 0; k < 3; ++k) ru[l][k] += w * gT[i] * xi[k];
                re[l] += 0.5 * w * (xi2 * gT[i] + hT[i]);
            }
        }
        for (int i = i0; i < i1; ++i) {
            int l = i - i0;
            o->rho[i] = rho[l];
            for (int k = 0; k < 3; ++k) o->U[3 * i + k] = ru[l][k] / rho[l];
            o->T[i] = (re[l] - 0.5 * rho[l] * magsqr3(o->U + 3 * i)) / (c1 * rho[l]);
            o->tau[i] = tau_of(o, o->T[i], o->rho[i]);
        }
        for (int v = 0; v < nV; ++v) {
            const double* xi = o->xi + 3 * v;
            const double w = o->w[v];
            const double* gT = o->gT + (size_t)v * nC;
            const double* hT = o->hT + (size_t)v * nC;
            for (int i = i0; i < i1; ++i) {
                int l = i - i0;
                double c[3] = {xi[0] - o->U[3 * i], xi[1] - o->U[3 * i + 1], xi[2] - o->U[3 * i + 2]};
                double s = magsqr3(c) * gT[i] + hT[i];
                for (int k = 0; k < 3; ++k) qq[l][k] += 0.5 * w * c[k] * s;
            }
        }
        for (int i = i0; i < i1; ++i) {
            int l = i - i0;
            double fac = 2.0 * o->tau[i] / (2.0 * o->tau[i] + dt * o->Pr);
            for (int k = 0; k < 3; ++k) o->q[3 * i + k] = fac * qq[l][k];
        }
    }
}

/* fvDVM::updateGHbarSurfSymmetryIn (fvDVM.C:375-454, discreteVelocity.C:733-817):
   incoming DVs (xi.S0 <= 0, S0 the patch's first face) of a symmetry patch
   take the face value of their mirror DV.  DVMsymmetry copies from a snapshot
   of all DVs taken before the pass; symmetryPlane copies DV by DV in DV order. */
static void symmetry_in(oracle_t* o) {
    const int nI = o->nI, nB = o->nB, nF = o->nF, nV = o->nV;
#pragma omp parallel
    {
        double* snap = (double*)malloc(sizeof(double) * 2 * (size_t)nV);
#pragma omp for schedule(dynamic, 4)
        for (int b = 0; b < nB; ++b) {
            const int kind = o->bKind[b];
            if (kind != ORACLE_PATCH_SYMMETRY_MOD && kind != ORACLE_PATCH_SYMMETRY_PLANE) continue;
            const int f = nI + b;
            const double* S0 = o->bS0 + 3 * b;
            for (int v = 0; v < nV; ++v) {
                snap[v] = o->gS[(size_t)v * nF + f];
                snap[nV + v] = o->hS[(size_t)v * nF + f];
            }
            for (int v = 0; v < nV; ++v) {
                if (!(dot3(o->xi + 3 * v, S0) <= 0)) continue;
                const int t = sym_target(o, v, S0);
                if (kind == ORACLE_PATCH_SYMMETRY_MOD) {
                    o->gS[(size_t)v * nF + f] = snap[t];
                    o->hS[(size_t)v * nF + f] = snap[nV + t];
                } else {
                    o->gS[(size_t)v * nF + f] = o->gS[(size_t)t * nF + f];
                    o->hS[(size_t)v * nF + f] = o->hS[(size_t)t * nF + f];
                }
            }
        }
        free(snap);
    }
}

/* fvDVM::updatePressureInOutBC (fvDVM.C:730-806), after the cell macros. */
static void pressure_bc(oracle_t* o) {
    const int nI = o->nI, nB = o->nB;
    const double R = o->R;
    for (int b = 0; b < nB; ++b) {
        const int kind = o->bKind[b];
        if (kind != ORACLE_PATCH_PRESSURE_IN && kind != ORACLE_PATCH_PRESSURE_OUT) continue;
        const int f = nI + b, P = o->bCell[b];
        const double* Sf = o->Sf + 3 * f;
        const double magSf = sqrt(magsqr3(Sf));
        const double n[3] = {Sf[0] / magSf, Sf[1] / magSf, Sf[2] / magSf};
        const double* Ui = o->U + 3 * P;
        const double Ti = o->T[P], rhoi = o->rho[P];
        const double ai = sqrt(R * Ti * (o->K + 5) / (o->K + 3));
        const double Un = dot3(Ui, n);
        double UnIn;
        if (kind == ORACLE_PATCH_PRESSURE_IN) {
            o->rhob[b] = o->pB[b] / R / o->Tb[b];
            UnIn = Un + (o->pB[b] - rhoi * R * Ti) / rhoi / ai;
        } else {
            o->rhob[b] = rhoi + (o->pB[b] - rhoi * R * Ti) / ai / ai;
            o->Tb[b] = o->pB[b] / (R * rhoi);
            UnIn = Un + (rhoi * R * Ti - o->pB[b]) / rhoi / ai;
        }
        for (int k = 0; k < 3; ++k) o->Ub[3 * b + k] = UnIn * n[k] + (Ui[k] - Un * n[k]);
    }
}

/* Uvol_.correctBoundaryConditions(); Tvol_.correctBoundaryConditions()
   (fvDVM.C:697-699, after the cell macros): a zeroGradient U or T patch takes
   its owner cell's value, which a farField or pressureIn patch then uses for
   its incoming Maxwellian and (pressureIn) its density p/(R T_b). */
static void zero_gradient_tu(oracle_t* o) {
    for (int b = 0; b < o->nB; ++b) {
        const int P = o->bCell[b];
        if (o->bZG[b] & 1) o->Tb[b] = o->T[P];
        if (o->bZG[b] & 2)
            for (int k = 0; k < 3; ++k) o->Ub[3 * b + k] = o->U[3 * P + k];
    }
}

/* fvDVM::evolution, fvDVM.C:1086-1108 */
static void evolution(oracle_t* o) {
    const int nV = o->nV, nC = o->nC, nB = o->nB, nI = o->nI, nF = o->nF;
#pragma omp parallel
    {
        double* grad = (double*)malloc(sizeof(double) * 3 * (size_t)nC);
        double* grh = (double*)malloc(sizeof(double) * 3 * (size_t)nC);
#pragma omp for schedule(dynamic, 1)
        for (int v = 0; v < nV; ++v) dv_bar_and_surf(o, v, grad, grh);
        free(grad);
        free(grh);
    }
    /* P4 fvDVM::updateMaxwellWallRho (fvDVM.C:347-367) ->
       calculatedMaxwellFvPatchField::evaluate (.C:140-164): outgoing flux
       accumulated in DV order, rho_w = outGoing/|inComingByRho|, reset. */
#pragma omp parallel for schedule(static)
    for (int b = 0; b < nB; ++b) {
        if (o->bKind[b] != ORACLE_PATCH_MAXWELL) continue;
        int f = nI + b;
        const double* S = o->Sf + 3 * f;
        double acc = o->outGoing[b];
        for (int v = 0; v < nV; ++v) {
            double xs = dot3(o->xi + 3 * v, S);
            if (xs > 0) acc += o->w[v] * xs * o->gS[(size_t)v * nF + f];
        }
        o->rhoW[b] = acc / fabs(o->inByRho[b]);
        o->outGoing[b] = 0.0;
    }
#pragma omp parallel for schedule(dynamic, 4)
    for (int v = 0; v < nV; ++v) dv_wall_in(o, v);
    symmetry_in(o);
    face_macros(o);
#pragma omp parallel for schedule(dynamic, 1)
    for (int v = 0; v < nV; ++v) dv_surf_and_tilde(o, v);
    cell_macros(o);
    zero_gradient_tu(o);
    pressure_bc(o);
}

void oracle_step(void* h, double dt, int nsteps) {
    oracle_t* o = (oracle_t*)h;
    o->dt = dt;
    for (int s = 0; s < nsteps; ++s) evolution(o);
}

void oracle_get_cell(void* h, double* rho, double* U, double* T, double* q, double* tau) {
    oracle_t* o = (oracle_t*)h;
    int n = o->nC;
    if (rho) memcpy(rho, o->rho, sizeof(double) * n);
    if (U) memcpy(U, o->U, sizeof(double) * 3 * n);
    if (T) memcpy(T, o->T, sizeof(double) * n);
    if (q) memcpy(q, o->q, sizeof(double) * 3 * n);
    if (tau) memcpy(tau, o->tau, sizeof(double) * n);
}

void oracle_get_face(void* h, double* rho, double* U, double* T, double* q, double* tau) {
    oracle_t* o = (oracle_t*)h;
    int n = o->nF;
    if (rho) memcpy(rho, o->rhoF, sizeof(double) * n);
    if (U) memcpy(U, o->UF, sizeof(double) * 3 * n);
    if (T) memcpy(T, o->TF, sizeof(double) * n);
    if (q) memcpy(q, o->qF, sizeof(double) * 3 * n);
    if (tau) memcpy(tau, o->tauF, sizeof(double) * n);
}

void oracle_get_wall(void* h, double* rhoW, double* qWall, double* stressWall) {
    oracle_t* o = (oracle_t*)h;
    int n = o->nB;
    if (rhoW) memcpy(rhoW, o->rhoW, sizeof(double) * n);
    if (qWall) memcpy(qWall, o->qWall, sizeof(double) * 3 * n);
    if (stressWall) memcpy(stressWall, o->stressWall, sizeof(double) * 9 * n);
}

void oracle_get_boundary(void* h, double* rhob, double* Ub, double* Tb) {
    oracle_t* o = (oracle_t*)h;
    int n = o->nB;
    if (rhob) memcpy(rhob, o->rhob, sizeof(double) * n);
    if (Ub) memcpy(Ub, o->Ub, sizeof(double) * 3 * n);
    if (Tb) memcpy(Tb, o->Tb, sizeof(double) * n);
}

void oracle_get_dist(void* h, double* g, double* hh) {
    oracle_t* o = (oracle_t*)h;
    size_t n = (size_t)o->nV * o->nC;
    if (g) memcpy(g, o->gT, sizeof(double) * n);
    if (hh) memcpy(hh, o->hT, sizeof(double) * n);
}

void oracle_set_dist(void* h, const double* g, const double* hh) {
    oracle_t* o = (oracle_t*)h;
    size_t n = (size_t)o->nV * o->nC;
    if (g) memcpy(o->gT, g, sizeof(double) * n);
    if (hh) memcpy(o->hT, hh, sizeof(double) * n);
}

void oracle_get_geometry(void* h, double* C, double* V, double* Cf, double* Sf, double* pVec, double* nVec,
                         double* bVec, double* deltaCoeffs) {
    oracle_t* o = (oracle_t*)h;
    if (C) memcpy(C, o->C, sizeof(double) * 3 * o->nC);
    if (V) memcpy(V, o->V, sizeof(double) * o->nC);
    if (Cf) memcpy(Cf, o->Cf, sizeof(double) * 3 * o->nF);
    if (Sf) memcpy(Sf, o->Sf, sizeof(double) * 3 * o->nF);
    if (pVec) memcpy(pVec, o->pVec, sizeof(double) * 3 * o->nI);
    if (nVec) memcpy(nVec, o->nVec, sizeof(double) * 3 * o->nI);
    if (bVec) memcpy(bVec, o->bVec, sizeof(double) * 3 * o->nB);
    if (deltaCoeffs) {
        memcpy(deltaCoeffs, o->dcI, sizeof(double) * o->nI);
        memcpy(deltaCoeffs + o->nI, o->dcB, sizeof(double) * o->nB);
    }
}

void oracle_get_dv(void* h, double* xi, double* w) {
    oracle_t* o = (oracle_t*)h;
    if (xi) memcpy(xi, o->xi, sizeof(double) * 3 * o->nV);
    if (w) memcpy(w, o->w, sizeof(double) * o->nV);
}

/* fvDVM::getCoNum, fvDVM.C:1111-1119 (internal faces only) */
void oracle_conum(void* h, double dt, double* maxCo, double* meanCo) {
    oracle_t* o = (oracle_t*)h;
    double mx = 0.0, sum = 0.0;
    for (int f = 0; f < o->nI; ++f) {
        double u = o->dcI[f] * (sqrt(magsqr3(o->UF + 3 * f)) + sqrt((double)o->D) * o->xiMax);
        if (u > mx || f == 0) mx = u;
        sum += u;
    }
    *maxCo = mx * dt;
    *meanCo = sum / o->nI * dt;
}
