/*
 * dugks_oracle.h -- TEST INFRASTRUCTURE ONLY.
 *
 * Plain-C FP64 restatement of dugksFoam's DUGKS time step (fvDVM::evolution,
 * src/fvDVM/fvDVM/fvDVM.C:1086-1108) used as the parity checker for the CUDA
 * engine and as the timed CPU baseline.  Only tests, the smoke check and the
 * benchmark's CPU leg may load it; the product never links it.
 *
 * Parity status: UNPINNED at the OpenFOAM boundary.  The reference ships no
 * tests, golden vectors or recorded outputs, and it cannot be built without
 * OpenFOAM + MPI.  The restatement follows the reference's operation order;
 * the OpenFOAM arithmetic it relies on (least-squares vectors, patch deltas,
 * fixedGradient evaluation, primitiveMesh geometry) is restated from
 * OpenFOAM >= 2.3 semantics and documented in dugks_oracle.c.
 */
#ifndef DUGKS_ORACLE_H
#define DUGKS_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Patch kinds understood by the oracle: the rho boundary-condition type,
   which discreteVelocity::setBCtype (discreteVelocity.C:250-300) maps to the
   g/h surface patch type given in brackets. */
enum {
    ORACLE_PATCH_EMPTY = 0,              /* "empty" (2D front/back) */
    ORACLE_PATCH_MAXWELL = 1,            /* "calculatedMaxwell" [maxwellWall] diffuse wall */
    ORACLE_PATCH_ZERO_GRADIENT = 2,      /* "zeroGradient" [zeroGradient] */
    ORACLE_PATCH_FIXED_VALUE = 3,        /* "fixedValue" [mixed]: incoming DFs frozen at the initial Maxwellian */
    ORACLE_PATCH_FAR_FIELD = 4,          /* "farField" [farField]: incoming DFs rho_b M(U_owner, T_b) */
    ORACLE_PATCH_PRESSURE_IN = 5,        /* "pressureIn" [farField] + fvDVM::updatePressureInOutBC */
    ORACLE_PATCH_PRESSURE_OUT = 6,       /* "pressureOut" [farField] + fvDVM::updatePressureInOutBC */
    ORACLE_PATCH_SYMMETRY_MOD = 7,       /* "symmetryMod" [DVMsymmetry]: mirrored DFs */
    ORACLE_PATCH_SYMMETRY_PLANE = 8      /* constraint "symmetryPlane": mirrored DFs */
};

typedef struct oracle_case {
    int nPoints;
    const double* points;                /* [nPoints][3] */
    int nCells, nFaces, nInternalFaces;
    const int* faceOffsets;              /* [nFaces+1] */
    const int* faceVerts;
    const int* owner;                    /* [nFaces] */
    const int* neighbour;                /* [nInternalFaces] */
    int nPatches;
    const int* patchStart;               /* [nPatches] global face index */
    const int* patchSize;
    const int* patchKind;                /* ORACLE_PATCH_* */
    const double* Ub;                    /* [nFaces-nInternalFaces][3] U patch values */
    const double* Tb;                    /* [nFaces-nInternalFaces]    T patch values */
    const double* rhob;                  /* [nFaces-nInternalFaces]    rho patch values (may be NULL) */
    const double* patchPressure;         /* [nPatches] pressureIn / pressureOut (may be NULL) */
    const int* patchTzg;                 /* [nPatches] 1: T boundary condition zeroGradient (may be NULL) */
    const int* patchUzg;                 /* [nPatches] 1: U boundary condition zeroGradient (may be NULL) */
    int nXiPerDim;
    const double* xis;                   /* [nXiPerDim] 1-D nodes  (constant/Xis) */
    const double* weights;               /* [nXiPerDim] 1-D weights (constant/weights) */
    double xiMax;                        /* DVMProperties fvDVMparas.xiMax */
    double R, omega, Tref, muRef, Pr;
    int KInner;
    const double* rho0;                  /* [nCells] */
    const double* U0;                    /* [nCells][3] */
    const double* T0;                    /* [nCells] */
} oracle_case;

void* oracle_create(const oracle_case* c);
void  oracle_destroy(void* h);
void  oracle_set_threads(int n);
int   oracle_nsolutiond(void* h);
int   oracle_ndv(void* h);
/* One or more DUGKS steps with a fixed dt (fvDVM::evolution per step). */
void  oracle_step(void* h, double dt, int nsteps);
void  oracle_get_cell(void* h, double* rho, double* U, double* T, double* q, double* tau);
/* Face macros for internal faces followed by every boundary face (empty ones zero). */
void  oracle_get_face(void* h, double* rho, double* U, double* T, double* q, double* tau);
/* Per boundary face: rho boundary value (Maxwell-wall density), qWall, stressWall[9]. */
void  oracle_get_wall(void* h, double* rhoW, double* qWall, double* stressWall);
/* Per boundary face: rho, U, T patch values (farField / pressure patches change them). */
void  oracle_get_boundary(void* h, double* rhob, double* Ub, double* Tb);
/* g~, h~ in DV-outer layout [nDV][nCells]. */
void  oracle_get_dist(void* h, double* g, double* hh);
void  oracle_set_dist(void* h, const double* g, const double* hh);
/* Geometry as the fv layer sees it (for host-geometry parity tests). */
void  oracle_get_geometry(void* h, double* C, double* V, double* Cf, double* Sf,
                          double* pVec, double* nVec, double* bVec, double* deltaCoeffs);
/* Discrete velocity set as built by fvDVM::initialiseDV. */
void  oracle_get_dv(void* h, double* xi, double* w);
/* fvDVM::getCoNum over internal faces with the current face velocity. */
void  oracle_conum(void* h, double dt, double* maxCo, double* meanCo);

#ifdef __cplusplus
}
#endif
#endif
