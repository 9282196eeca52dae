/*
 * dugks.h -- C ABI of the GB300 DUGKS time-step engine.
 *
 * Drop-in for the per-time-step engine of dugksFoam, class Foam::fvDVM
 * (src/fvDVM/fvDVM/fvDVM.H:78-377).  Each entry point names the reference
 * interface it replaces.  Plain pointers and sizes only; every call returns
 * an int status (0 = DUGKS_OK); dugks_last_error() gives the message.
 *
 * Ownership: all host pointers passed in are caller-owned and copied during
 * the call.  Device memory is owned by the handle.  A handle is not
 * thread-safe; separate handles on separate streams are independent.
 *
 * Units and layouts (SI, as in the reference):
 *   cell fields   rho[nCells], U[nCells][3], T[nCells], q[nCells][3]
 *   face indices  internal faces 0..nInternal-1 then boundary faces in
 *                 OpenFOAM order (patch by patch)
 *   distribution  g[nCells][nDV] (DV index innermost; DV i = iz*M*M+iy*M+ix)
 */
#ifndef DUGKS_DUGKS_H
#define DUGKS_DUGKS_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define DUGKS_ABI_VERSION 3

typedef struct dugks_handle dugks_handle;

enum dugks_status {
    DUGKS_OK = 0,
    DUGKS_ERR_ARG = 1,          /* invalid argument / inconsistent case   */
    DUGKS_ERR_IO = 2,           /* case-directory parse or file error     */
    DUGKS_ERR_UNSUPPORTED = 3,  /* boundary type or layout not supported  */
    DUGKS_ERR_CUDA = 4,         /* CUDA runtime error / no device         */
    DUGKS_ERR_NUMERIC = 5,      /* NaN/Inf or non-positive rho or T found */
    DUGKS_ERR_TIMEOUT = 6,      /* a bounded device wait gave up          */
    DUGKS_ERR_OOM = 7,          /* device allocation failed               */
    DUGKS_ERR_BOUNDS = 8        /* checked build: an index read from mesh
                                   or tile data was out of range           */
};

/* 1 in the checked build (libdugks_checked.so: device-side index checks that
 * report DUGKS_ERR_BOUNDS instead of reading out of range), else 0. */
int dugks_checked_build(void);

/* Storage/arithmetic precision of the distributions. */
enum dugks_precision {
    DUGKS_FP64 = 0,             /* plain FP64 everywhere                         */
    DUGKS_FP32_FP64MOM = 1      /* FP32 g,h/reconstruction/fluxes; FP64 moments  */
};

/* Patch kinds: the rho boundary-condition type of 0/rho
 * (discreteVelocity::setBCtype, discreteVelocity.C:250-300, maps it to the
 * g/h surface patch type given in brackets).  Every kind runs on the plain
 * FP64 pipeline (DUGKS_FP64 with DUGKS_PIPE_REFERENCE or AUTO) and on the FP32
 * pipeline (DUGKS_FP32_FP64MOM); the fused FP64 sweeps, the batched kernels
 * and the gradient harness take diffuse walls and empty patches only. */
enum dugks_patch_kind {
    DUGKS_PATCH_EMPTY = 0,          /* "empty" (2D front/back)                            */
    DUGKS_PATCH_MAXWELL = 1,        /* "calculatedMaxwell" [maxwellWall] diffuse wall     */
    DUGKS_PATCH_ZERO_GRADIENT = 2,  /* "zeroGradient" [zeroGradient]: face = owner cell   */
    DUGKS_PATCH_FIXED_VALUE = 3,    /* "fixedValue" [mixed]: incoming DFs stay at the
                                       Maxwellian of the initial patch rho, U, T          */
    DUGKS_PATCH_FAR_FIELD = 4,      /* "farField" [farField]: incoming DFs
                                       rho_b M(U of the owner cell, T_b)                  */
    DUGKS_PATCH_PRESSURE_IN = 5,    /* "pressureIn" [farField]; rho_b = p/(R T_b) at
                                       creation and after each step
                                       (fvDVM::updatePressureInOutBC)                     */
    DUGKS_PATCH_PRESSURE_OUT = 6,   /* "pressureOut" [farField]; rho_b, T_b from p and
                                       the owner cell, at creation and after each step    */
    DUGKS_PATCH_SYMMETRY_MOD = 7,   /* "symmetryMod" [DVMsymmetry]: incoming DFs mirror
                                       the outgoing ones                                  */
    DUGKS_PATCH_SYMMETRY_PLANE = 8  /* constraint "symmetryPlane": mirrored incoming DFs  */
};

/* Kernel pipeline selection (both produce the same step). */
enum dugks_pipeline {
    DUGKS_PIPE_AUTO = 0,        /* fused tile sweeps when supported              */
    DUGKS_PIPE_REFERENCE = 1,   /* one kernel per reference pass                 */
    DUGKS_PIPE_FUSED = 2        /* two fused tile sweeps per step                */
};

/* In-memory case: replaces the constructor
 *   fvDVM(volScalarField& rho, volVectorField& U, volScalarField& T,
 *         int* argc, char*** argv, argList& args)     fvDVM.C:886-1075
 * plus the mesh, constant/DVMProperties, constant/Xis, constant/weights and
 * the 0/{rho,U,T} boundary values it reads. */
typedef struct dugks_case_desc {
    int32_t n_points;
    const double* points;            /* [n_points][3]                        */
    int32_t n_cells, n_faces, n_internal_faces;
    const int32_t* face_offsets;     /* [n_faces+1] CSR into face_verts      */
    const int32_t* face_verts;
    const int32_t* owner;            /* [n_faces]                            */
    const int32_t* neighbour;        /* [n_internal_faces]                   */
    int32_t n_patches;
    const int32_t* patch_start;      /* [n_patches] global face index        */
    const int32_t* patch_size;
    const int32_t* patch_kind;       /* dugks_patch_kind                     */
    const double* wall_U;            /* [n_faces-n_internal_faces][3] U patch values */
    const double* wall_T;            /* [n_faces-n_internal_faces]    T patch values */
    const double* bnd_rho;           /* [n_faces-n_internal_faces] rho patch values
                                        (fixedValue, farField); NULL if unused       */
    const double* patch_pressure;    /* [n_patches] pressureIn / pressureOut values;
                                        NULL if unused                               */
    int32_t n_xi_per_dim;            /* fvDVMparas.nDV                       */
    const double* xis;               /* [n_xi_per_dim] constant/Xis          */
    const double* weights;           /* [n_xi_per_dim] constant/weights      */
    double xi_max;                   /* fvDVMparas.xiMax                     */
    double R, omega, Tref, muRef, Pr;/* gasProperties                        */
    int32_t KInner;
    const double* rho0;              /* [n_cells] initial fields (0/rho ...) */
    const double* U0;                /* [n_cells][3]                         */
    const double* T0;                /* [n_cells]                            */
    int32_t precision;               /* dugks_precision                      */
    int32_t pipeline;                /* dugks_pipeline                       */
    int32_t device;                  /* CUDA device ordinal                  */
    /* ABI version 3: per patch, 1 when the T (U) boundary condition is
     * zeroGradient, else 0; NULL: none.  Such a patch takes the owner cells'
     * initial values at creation and their new values after every step
     * (Tvol_/Uvol_.correctBoundaryConditions(), fvDVM.C:697-699), before the
     * pressure-patch update; a farField or pressureIn patch then uses that T
     * for its incoming Maxwellian (and pressureIn for rho_b = p/(R T_b)).
     * Refused (DUGKS_ERR_UNSUPPORTED) on diffuse-wall patches. */
    const int32_t* patch_T_zero_gradient;
    const int32_t* patch_U_zero_gradient;
} dugks_case_desc;

typedef struct dugks_info {
    /* n_wall_faces: every non-empty boundary face (walls and the other types);
     * dugks_get_face_macros covers the internal faces followed by these */
    int32_t n_cells, n_faces, n_internal_faces, n_wall_faces;
    int32_t n_dv, n_dv_padded, n_solution_d, has_h;
    int32_t precision, pipeline;
    double dt;
    int64_t step_count;
    size_t device_bytes;             /* device memory held by the handle     */
    /* fvDVM accessors nXiPerDim(), KInner(), xiMax(), R(), omega(), Tref(),
     * muRef(), Pr() (fvDVMI.H:97-155) */
    int32_t n_xi_per_dim, KInner;
    double xi_max, R, omega, Tref, muRef, Pr;
} dugks_info;

/* fvDVM::fvDVM (fvDVM.C:886-1075): build the engine from an in-memory case.
 * g~,h~ start at the Shakhov equilibrium of (rho0,U0,T0,q=0)
 * (discreteVelocity::initDFtoEq, discreteVelocity.C:220-249). */
int dugks_create(const dugks_case_desc* desc, dugks_handle** out);

/* fvDVM::fvDVM from an OpenFOAM case directory: constant/polyMesh/{points,faces,owner,neighbour,boundary},
 * constant/DVMProperties, constant/Xis, constant/weights, 0/{rho,U,T},
 * system/controlDict (deltaT).  rho patch types supported: empty,
 * calculatedMaxwell, zeroGradient, fixedValue, farField, pressureIn,
 * pressureOut, symmetryMod and the symmetryPlane constraint (dugks_patch_kind);
 * any other type fails with DUGKS_ERR_UNSUPPORTED. */
int dugks_create_from_case_dir(const char* case_dir, int32_t precision, dugks_handle** out);

int dugks_destroy(dugks_handle* h);
const char* dugks_last_error(const dugks_handle* h);   /* never NULL */
const char* dugks_global_error(void);                  /* last create failure */
int dugks_get_info(dugks_handle* h, dugks_info* info);

/* Time::setDeltaT as driven by setDeltaTvar.H:34-50. */
int dugks_set_dt(dugks_handle* h, double dt);
int dugks_get_dt(dugks_handle* h, double* dt);

/* Run the CUDA work of this handle on an existing stream (cudaStream_t);
 * NULL restores the handle's own stream. */
int dugks_set_stream(dugks_handle* h, void* stream);

/* fvDVM::evolution() (fvDVM.C:1086-1108) n times.  Asynchronous on the
 * handle's stream; the NaN/negative-state check runs on the device and is
 * reported by the next synchronising call (get_* / dugks_synchronize). */
int dugks_step(dugks_handle* h, int32_t nsteps);
int dugks_synchronize(dugks_handle* h);

/* fvDVM::getCoNum (fvDVM.C:1111-1119): max and mean Courant number over
 * internal faces with the current face velocity. */
int dugks_get_conum(dugks_handle* h, double* max_co, double* mean_co);

/* Accessors rhoVol(), Uvol(), Tvol(), qVol(), tauVol() (fvDVMI.H:26-155).
 * Any pointer may be NULL.  The copies are queued behind the handle's
 * stream and finished by one wait; when that wait reports an error of a
 * previous step (DUGKS_ERR_NUMERIC, ...), the buffers hold that step's values. */
int dugks_get_macros(dugks_handle* h, double* rho, double* U, double* T, double* q, double* tau);

/* rhoSurf(), Usurf(), Tsurf(), qSurf(), tauSurf() for internal faces then
 * wall faces (face order); empty-patch faces are not stored.  Any may be NULL. */
int dugks_get_face_macros(dugks_handle* h, double* rho, double* U, double* T, double* q, double* tau);

/* Boundary state of one patch (patch index as in the case): Maxwell-wall
 * density rho_w (calculatedMaxwellFvPatchField value), qWall[3] and
 * stressWall[9] per face (fvDVM.C:539-581).  Any pointer may be NULL. */
int dugks_get_wall(dugks_handle* h, int32_t patch, double* rho_w, double* q_wall, double* stress_wall);

/* Patch values of the volume fields rhoVol(), Uvol(), Tvol() on one non-empty
 * patch (fvDVMI.H:26-60 boundaryField()): rho is the Maxwell-wall density on
 * walls and the rho patch value elsewhere (pressureIn / pressureOut patches
 * change rho, U and T after each step, fvDVM.C:730-806).  rho[n], U[n][3],
 * T[n] for the patch's n faces; any pointer may be NULL. */
int dugks_get_boundary(dugks_handle* h, int32_t patch, double* rho, double* U, double* T);

/* Steady-state residuals of dugksFoam.C:88-107: sum|U-Uold|/sum|U|,
 * sum|T-Told|/sum T, sum|rho-rhoOld|/sum rho against the fields saved by the
 * previous call (or creation); then saves the current fields.
 * res = {Uchange, TemperatureChange, rhoChange}. */
int dugks_get_residual(dugks_handle* h, double res[3]);

/* Distribution functions g~, h~ as FP64 [n_cells][n_dv] (h may be NULL).
 * gTildeVol()/hTildeVol() of every discreteVelocity (discreteVelocity.H:85-103). */
int dugks_get_dist(dugks_handle* h, double* g, double* hh);
int dugks_set_dist(dugks_handle* h, const double* g, const double* hh);

/* Exact-restart checkpoint: g~, h~, lagged boundary gradients, cell macros,
 * face velocities and dt.  The reference restarts inexactly (g~ is NO_WRITE,
 * discreteVelocity.C:76-83); this fixes it. */
int dugks_checkpoint_size(dugks_handle* h, size_t* bytes);
int dugks_checkpoint_save(dugks_handle* h, void* buf, size_t bytes);
int dugks_checkpoint_load(dugks_handle* h, const void* buf, size_t bytes);

/* Per-kernel device time of one step, measured with CUDA events around each
 * launch over nsteps steps (blocking).  names receives a '\n'-separated list;
 * ms[i] is the mean per-step time of kernel i. */
int dugks_profile_step(dugks_handle* h, int32_t nsteps, char* names, size_t names_len,
                       double* ms, int32_t max_kernels, int32_t* n_kernels);

/* Number of kernel launches one dugks_step(h, 1) issues. */
int dugks_launches_per_step(dugks_handle* h, int32_t* n);

/* Cell macros rho, U, T, q of distributions the caller holds on the device,
 * computed without allocating any memory.  No counterpart in the reference:
 * it is for callers that cannot allocate device memory where they need it --
 * code inside a runtime that owns every device allocation, or a time loop
 * that must not call cudaMalloc/cudaFree (they synchronise the device).
 * g, hh: device arrays [n_cells][n_dv] in FP64 (the dugks_get_dist layout;
 * hh may be NULL when the case has no h).  rho[n_cells], U[n_cells][3],
 * T[n_cells], q[n_cells][3]: device output arrays (any may be NULL).  Uses the
 * handle's velocity set, gas properties and dt (q is scaled by
 * 2 tau/(2 tau + dt Pr) as in updateMacroVol, fvDVM.C:597-728) and runs
 * asynchronously on the handle's stream; the caller orders its own writes of
 * g/hh before the call and reads the outputs after dugks_synchronize.
 * Scratch is a static device array shared by all calls: at most 262144 cells
 * (larger cases are rejected with DUGKS_ERR_ARG); calls whose work overlaps on
 * the GPU race.  The first call on each device looks up the array's device
 * address (cudaGetSymbolAddress) and caches it for the process; make that
 * first call before any stream capture, and none after a cudaDeviceReset.
 * The caller's current device is left as it was; a CUDA error pending from
 * the caller's earlier work is reported (DUGKS_ERR_CUDA) without launching;
 * n_cells == 0 returns DUGKS_OK without launching. */
int dugks_macros_noalloc(dugks_handle* h, const double* g, const double* hh, double* rho, double* U, double* T,
                         double* q);

/* Sizes and parameters of an OpenFOAM case directory, read on the host only
 * (no device, no handle): the same reader as dugks_create_from_case_dir. */
typedef struct dugks_case_summary {
    int32_t n_points, n_cells, n_faces, n_internal_faces, n_patches, n_wall_faces, n_empty_faces;
    int32_t n_xi_per_dim, KInner;
    double xi_max, R, omega, Tref, muRef, Pr, delta_t;
    double rho_sum, T_sum;          /* sums of the 0/rho and 0/T internal fields */
    int32_t n_df_cells;             /* length of DVMProperties DFwriteCellList   */
} dugks_case_summary;
int dugks_inspect_case_dir(const char* case_dir, dugks_case_summary* out);

/* fvDVM::writeDFonCells (fvDVM.C:820-882, called by dugksFoam.C:78 at output
 * times): for each cell id, the file <case_dir>/0/DF<id> (an OpenFOAM
 * scalarList of n_dv values) holding g~ of that cell over the velocity set.
 * cells == NULL takes DFwriteCellList of the case directory the handle was
 * created from (nothing to do when it has none). */
int dugks_write_df_on_cells(dugks_handle* h, const char* case_dir, const int32_t* cells, int32_t n_cells);

/* runTime.write() of dugksFoam.C:81: write the current fields into
 * <case_dir>/<time_name>/ in OpenFOAM ASCII (17 significant digits):
 * rho, U, T (createFields.H AUTO_WRITE), q (fvDVM qVol_), qSurf and
 * stressSurf (fvDVM qWall_/stressWall_: zero internal field, wall heat flux
 * and stress on the wall patches).  Wall patches of rho keep the
 * calculatedMaxwell type with the wall density as value, U and T are
 * fixedValue with the wall velocity and temperature, so a written time
 * directory is a valid 0/ for dugks_create_from_case_dir.  Patch names are
 * those of the case directory, or patch<i> for handles made by dugks_create. */
int dugks_write_time(dugks_handle* h, const char* case_dir, const char* time_name);

/* ---- gradient harness (no counterpart in the reference) ----
 * Objective over a window of FP64 steps from the handle's initial state:
 *   J = 1/(n_steps-avg_first) * sum_{n=avg_first}^{n_steps-1}
 *       [ sum_{w in q_patch} S_w . qWall_w(n) + sum_{w in stress_patch} |S_w| stressWall_w,xy(n) ]
 * (qWall, stressWall as fvDVM::updateMacroSurf, fvDVM.C:535-576).  Parameters:
 * the wall temperature of every wall face (wall order = patch order) and the
 * viscosity scale s (mu_ref -> s mu_ref, derivatives at s = 1).  These run the
 * plain FP64 reference pipeline on private buffers; the handle's state, dt
 * and stream are used but its fields are not modified. */
typedef struct dugks_objective {
    int32_t n_steps, avg_first;
    int32_t q_patch, stress_patch;   /* patch indices, -1 for an absent term */
    int32_t checkpoint_every;        /* adjoint: steps between stored states */
} dugks_objective;

int dugks_objective_value(dugks_handle* h, const dugks_objective* o, double* J);
/* Tangent-linear (forward-mode) derivative along (dTw [n_wall_faces], ds). */
int dugks_objective_tangent(dugks_handle* h, const dugks_objective* o, const double* dTw, double ds, double* J,
                            double* dJ);
/* Adjoint gradient: dJ/dTw [n_wall_faces] and dJ/ds, with J. */
int dugks_objective_adjoint(dugks_handle* h, const dugks_objective* o, double* J, double* dJ_dTw, double* dJ_ds);

/* ---- batched cases (no counterpart in the reference) ----
 * Independent 2D cases (uneven meshes and velocity grids) advanced together
 * with the FP32 pipeline: every pass of the step is one launch over all cases,
 * the cases are split into groups whose launch chains are independent
 * branches of one CUDA graph (two steps per graph, replayed); or the
 * persistent kernel (groups -1): every pass of every step of every case in
 * one cooperative launch per dugks_batch_step, the passes separated by
 * grid-wide barriers whose waits give up after a bounded number of polls
 * (dugks_batch_synchronize then returns DUGKS_ERR_TIMEOUT).  autotune 1: the
 * DVs per lane (2 or 4), the cap on cells per tile and the number of groups
 * (0: every case its own graph branch with its own kernels; -1: persistent)
 * are chosen by timing a few steps of each candidate; 0: 4 DVs per lane, no
 * cap, one group; 2: the persistent kernel.  Cases with boundary types other
 * than diffuse walls run each with its own kernels as a branch of the graph
 * (groups 0; chosen by autotune 0 and 1, refused by 2).  Each case starts
 * from its own initial state; set each case's dt before stepping. */
typedef struct dugks_batch dugks_batch;
typedef struct dugks_batch_info {
    int32_t n_cases, dv_per_lane, tile_cap, groups, launches_per_step /* kernel nodes per step */, steps_per_graph,
        n_tuned;
    int64_t cells, cell_dv;               /* summed over the cases (cell*DV uses unpadded DVs) */
    int32_t tuned_dv_per_lane[8], tuned_tile_cap[8], tuned_groups[8];
    double tuned_ms_per_step[8];          /* timing of each candidate */
} dugks_batch_info;

int dugks_batch_create(const dugks_case_desc* descs, int32_t n_cases, int32_t autotune, dugks_batch** out);
int dugks_batch_destroy(dugks_batch* b);
const char* dugks_batch_last_error(const dugks_batch* b);
int dugks_batch_set_dt(dugks_batch* b, int32_t i, double dt);
int dugks_batch_step(dugks_batch* b, int32_t nsteps);      /* asynchronous */
int dugks_batch_synchronize(dugks_batch* b);
int dugks_batch_get_macros(dugks_batch* b, int32_t i, double* rho, double* U, double* T, double* q);
int dugks_batch_get_info(dugks_batch* b, dugks_batch_info* out);
/* Polls a grid-barrier wait of the persistent kernel makes before it gives up
 * (default 2^24, about a second); 0 makes every wait that has to wait give up. */
int dugks_batch_set_wait_limit(dugks_batch* b, int64_t polls);

#ifdef __cplusplus
}
#endif
#endif
