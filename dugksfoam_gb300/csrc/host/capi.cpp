// extern "C" entry points of libdugks (include/dugks/dugks.h).
#include <cstring>
#include <exception>
#include <cstdio>
#include <filesystem>
#include <memory>
#include <string>
#include <vector>

#include "../cuda/noalloc.h"
#include "dugks/dugks.h"
#include "foam_io.h"
#include "objective.h"
#include "batch.h"
#include "solver.h"

struct dugks_handle {
    std::unique_ptr<dugks::Solver> solver;
    std::string err;
    // case description kept on the host for dugks_write_time
    std::vector<std::string> patchNames;
    std::vector<int32_t> patchStart, patchSize, patchKind;
    std::vector<double> wallU, wallT;  // per boundary face
    std::vector<double> patchPressure; // per patch (pressureIn / pressureOut)
    std::vector<int32_t> patchTzg, patchUzg;  // per patch: T / U zeroGradient
    std::vector<int32_t> dfCells;      // DFwriteCellList of the case directory
};

namespace {
thread_local std::string g_err;

int guard(dugks_handle* h, int rc) {
    if (h && rc != DUGKS_OK && h->solver) h->err = h->solver->error();
    return rc;
}

template <typename F>
int call(dugks_handle* h, F&& f) {
    if (!h || !h->solver) return DUGKS_ERR_ARG;
    try {
        return guard(h, f(*h->solver));
    } catch (const std::exception& e) {
        h->err = e.what();
        return DUGKS_ERR_ARG;
    } catch (...) {
        h->err = "unknown exception";
        return DUGKS_ERR_ARG;
    }
}
}  // namespace

extern "C" {

int dugks_create(const dugks_case_desc* desc, dugks_handle** out) {
    if (!desc || !out) { g_err = "null argument"; return DUGKS_ERR_ARG; }
    *out = nullptr;
    try {
        std::string err;
        int code = DUGKS_OK;
        auto s = dugks::Solver::create(*desc, err, code);
        if (!s) { g_err = err; return code; }
        auto* h = new dugks_handle{std::move(s), std::string(), {}, {}, {}, {}, {}, {}, {}, {}, {}, {}};
        const int nB = desc->n_faces - desc->n_internal_faces;
        for (int p = 0; p < desc->n_patches; ++p) {
            h->patchNames.push_back("patch" + std::to_string(p));
            h->patchStart.push_back(desc->patch_start[p]);
            h->patchSize.push_back(desc->patch_size[p]);
            h->patchKind.push_back(desc->patch_kind[p]);
        }
        if (desc->wall_U) h->wallU.assign(desc->wall_U, desc->wall_U + 3 * (size_t)nB);
        if (desc->wall_T) h->wallT.assign(desc->wall_T, desc->wall_T + nB);
        if (desc->patch_pressure) h->patchPressure.assign(desc->patch_pressure, desc->patch_pressure + desc->n_patches);
        h->patchTzg.assign(desc->n_patches, 0);
        h->patchUzg.assign(desc->n_patches, 0);
        for (int p = 0; p < desc->n_patches; ++p) {
            if (desc->patch_T_zero_gradient) h->patchTzg[p] = desc->patch_T_zero_gradient[p];
            if (desc->patch_U_zero_gradient) h->patchUzg[p] = desc->patch_U_zero_gradient[p];
        }
        *out = h;
        return DUGKS_OK;
    } catch (const std::exception& e) {
        g_err = e.what();
        return DUGKS_ERR_ARG;
    }
}

int dugks_create_from_case_dir(const char* dir, int32_t precision, dugks_handle** out) {
    if (!dir || !out) { g_err = "null argument"; return DUGKS_ERR_ARG; }
    *out = nullptr;
    dugks::FoamCase c;
    std::string err;
    if (!dugks::read_foam_case(dir, c, err)) {
        g_err = err;
        return err.find("unsupported") != std::string::npos ? DUGKS_ERR_UNSUPPORTED : DUGKS_ERR_IO;
    }
    dugks_case_desc d{};
    d.n_points = (int32_t)(c.points.size() / 3);
    d.points = c.points.data();
    d.n_cells = c.nCells; d.n_faces = c.nFaces; d.n_internal_faces = c.nInternal;
    d.face_offsets = c.faceOffsets.data(); d.face_verts = c.faceVerts.data();
    d.owner = c.owner.data(); d.neighbour = c.neighbour.data();
    d.n_patches = (int32_t)c.patchNames.size();
    d.patch_start = c.patchStart.data(); d.patch_size = c.patchSize.data(); d.patch_kind = c.patchKind.data();
    d.wall_U = c.wallU.data(); d.wall_T = c.wallT.data();
    d.bnd_rho = c.bndRho.data(); d.patch_pressure = c.patchPressure.data();
    d.patch_T_zero_gradient = c.patchTzg.data(); d.patch_U_zero_gradient = c.patchUzg.data();
    d.n_xi_per_dim = c.nDV; d.xis = c.xis.data(); d.weights = c.weights.data(); d.xi_max = c.xiMax;
    d.R = c.R; d.omega = c.omega; d.Tref = c.Tref; d.muRef = c.muRef; d.Pr = c.Pr; d.KInner = c.KInner;
    d.rho0 = c.rho0.data(); d.U0 = c.U0.data(); d.T0 = c.T0.data();
    d.precision = precision;
    d.pipeline = DUGKS_PIPE_AUTO;
    d.device = 0;
    int rc = dugks_create(&d, out);
    if (rc == DUGKS_OK) (*out)->patchNames = c.patchNames;
    if (rc == DUGKS_OK) (*out)->dfCells = c.dfCells;
    if (rc == DUGKS_OK && c.deltaT > 0) (*out)->solver->setDt(c.deltaT);
    return rc;
}

int dugks_inspect_case_dir(const char* dir, dugks_case_summary* out) {
    if (!dir || !out) { g_err = "null argument"; return DUGKS_ERR_ARG; }
    dugks::FoamCase c;
    std::string err;
    if (!dugks::read_foam_case(dir, c, err)) {
        g_err = err;
        return err.find("unsupported") != std::string::npos ? DUGKS_ERR_UNSUPPORTED : DUGKS_ERR_IO;
    }
    dugks_case_summary r{};
    r.n_points = (int32_t)(c.points.size() / 3);
    r.n_cells = c.nCells; r.n_faces = c.nFaces; r.n_internal_faces = c.nInternal;
    r.n_patches = (int32_t)c.patchNames.size();
    r.n_df_cells = (int32_t)c.dfCells.size();
    for (size_t p = 0; p < c.patchNames.size(); ++p) {
        if (c.patchKind[p] == DUGKS_PATCH_MAXWELL) r.n_wall_faces += c.patchSize[p];
        if (c.patchKind[p] == DUGKS_PATCH_EMPTY) r.n_empty_faces += c.patchSize[p];
    }
    r.n_xi_per_dim = c.nDV; r.KInner = c.KInner;
    r.xi_max = c.xiMax; r.R = c.R; r.omega = c.omega; r.Tref = c.Tref; r.muRef = c.muRef; r.Pr = c.Pr;
    r.delta_t = c.deltaT;
    for (double v : c.rho0) r.rho_sum += v;
    for (double v : c.T0) r.T_sum += v;
    *out = r;
    return DUGKS_OK;
}

int dugks_write_df_on_cells(dugks_handle* h, const char* case_dir, const int32_t* cells, int32_t n_cells) {
    if (!h || !h->solver || !case_dir || (cells && n_cells < 0)) return DUGKS_ERR_ARG;
    return call(h, [&](dugks::Solver& s) -> int {
        std::vector<int32_t> ids = cells ? std::vector<int32_t>(cells, cells + n_cells) : h->dfCells;
        if (ids.empty()) return DUGKS_OK;
        const int nC = s.mesh().nC;
        for (int32_t id : ids)
            if (id < 0 || id >= nC) return s.fail(DUGKS_ERR_ARG, "write_df_on_cells: cell out of range");
        dugks_info info{};
        s.info(info);
        const size_t nV = (size_t)info.n_dv;
        std::vector<double> g((size_t)nC * nV);
        if (int e = s.getDist(g.data(), nullptr)) return e;
        const std::string dir = std::string(case_dir) + "/0";
        std::error_code ec;
        std::filesystem::create_directories(dir, ec);
        if (ec) return s.fail(DUGKS_ERR_IO, "cannot create " + dir + ": " + ec.message());
        for (int32_t id : ids) {
            std::string err;
            const std::string name = "DF" + std::to_string(id);
            if (!dugks::write_scalar_list(dir + "/" + name, name, g.data() + (size_t)id * nV, (int)nV, err))
                return s.fail(DUGKS_ERR_IO, err);
        }
        return DUGKS_OK;
    });
}

int dugks_write_time(dugks_handle* h, const char* case_dir, const char* time_name) {
    if (!h || !h->solver || !case_dir || !time_name) return DUGKS_ERR_ARG;
    return call(h, [&](dugks::Solver& s) -> int {
        const dugks::Mesh& m = s.mesh();
        const int nC = m.nC, nI = m.nI, nP = (int)h->patchNames.size();
        std::vector<double> rho(nC), U(3 * (size_t)nC), T(nC), q(3 * (size_t)nC);
        if (int e = s.macros(rho.data(), U.data(), T.data(), q.data(), nullptr)) return e;
        std::vector<double> qF(3 * (size_t)(m.nI + m.nW));
        if (int e = s.faceMacros(nullptr, nullptr, nullptr, qF.data(), nullptr)) return e;
        // per patch outputs, in patch face order
        static const char* const kRhoType[] = {"empty", "calculatedMaxwell", "zeroGradient", "fixedValue", "farField",
                                               "pressureIn", "pressureOut", "symmetryMod", "symmetryPlane"};
        std::vector<dugks::PatchOut> pr(nP), pu(nP), pt(nP), pq(nP), pqs(nP), pst(nP);
        for (int p = 0; p < nP; ++p) {
            const int kind = h->patchKind[p];
            const bool wall = kind == DUGKS_PATCH_MAXWELL, empty = kind == DUGKS_PATCH_EMPTY;
            const bool plane = kind == DUGKS_PATCH_SYMMETRY_PLANE;
            const char* uT = empty ? "empty" : (plane ? "symmetryPlane" : "fixedValue");
            const char* calc = empty ? "empty" : (plane ? "symmetryPlane" : "calculated");
            pr[p] = {h->patchNames[p], kRhoType[kind], {}, {}};
            pu[p] = {h->patchNames[p], uT, {}, {}};
            pt[p] = pu[p];
            // zeroGradient U / T patches are written as such (their value follows the owner)
            if (!empty && !plane && !h->patchUzg.empty() && h->patchUzg[p]) pu[p].type = "zeroGradient";
            if (!empty && !plane && !h->patchTzg.empty() && h->patchTzg[p]) pt[p].type = "zeroGradient";
            pq[p] = {h->patchNames[p], calc, {}, {}};
            pqs[p] = pq[p];
            pst[p] = pq[p];
            if (empty || plane) continue;
            const int n = h->patchSize[p];
            if (kind == DUGKS_PATCH_PRESSURE_IN || kind == DUGKS_PATCH_PRESSURE_OUT) {
                char buf[64];
                std::snprintf(buf, sizeof buf, "%.17g", h->patchPressure.empty() ? 0.0 : h->patchPressure[p]);
                pr[p].extra = std::string(kRhoType[kind]) + " " + buf;
            }
            std::vector<double> rb(n), ub(3 * (size_t)n), tb(n), qw(3 * (size_t)n, 0.0), sw(9 * (size_t)n, 0.0);
            if (int e = s.boundary(p, rb.data(), ub.data(), tb.data())) return e;
            if (wall && (s.wall(p, nullptr, qw.data(), sw.data()) != DUGKS_OK)) return DUGKS_ERR_CUDA;
            if (kind == DUGKS_PATCH_ZERO_GRADIENT || kind == DUGKS_PATCH_SYMMETRY_MOD)
                for (int i = 0; i < n; ++i) rb[i] = rho[m.owner[h->patchStart[p] + i]];
            pr[p].values = rb;
            pu[p].values = ub;
            pt[p].values = tb;
            pqs[p].values = qw;
            pst[p].values = sw;
        }
        // face heat flux of the active boundary faces, by boundary index -> patch position
        for (int p = 0; p < nP; ++p)
            if (h->patchKind[p] != DUGKS_PATCH_EMPTY && h->patchKind[p] != DUGKS_PATCH_SYMMETRY_PLANE)
                pq[p].values.assign(3 * (size_t)h->patchSize[p], 0.0);
        for (int w = 0; w < m.nW; ++w) {
            const int p = m.wallPatch[w], i = m.wallFace[w] - h->patchStart[p];
            if (pq[p].values.empty()) continue;
            for (int k = 0; k < 3; ++k) pq[p].values[3 * (size_t)i + k] = qF[3 * (size_t)(nI + w) + k];
        }
        const std::string dir = std::string(case_dir) + "/" + time_name;
        std::error_code ec;
        std::filesystem::create_directories(dir, ec);
        if (ec) return s.fail(DUGKS_ERR_IO, "cannot create " + dir + ": " + ec.message());
        std::string err;
        const bool ok =
            dugks::write_vol_field(dir + "/rho", "rho", "[1 -3 0 0 0 0 0]", 1, rho.data(), nC, pr, err) &&
            dugks::write_vol_field(dir + "/U", "U", "[0 1 -1 0 0 0 0]", 3, U.data(), nC, pu, err) &&
            dugks::write_vol_field(dir + "/T", "T", "[0 0 0 1 0 0 0]", 1, T.data(), nC, pt, err) &&
            dugks::write_vol_field(dir + "/q", "q", "[1 0 -3 0 0 0 0]", 3, q.data(), nC, pq, err) &&
            dugks::write_vol_field(dir + "/qSurf", "qSurf", "[1 0 -3 0 0 0 0]", 3, nullptr, nC, pqs, err) &&
            dugks::write_vol_field(dir + "/stressSurf", "stressSurf", "[1 -1 -2 0 0 0 0]", 9, nullptr, nC, pst, err);
        if (!ok) return s.fail(DUGKS_ERR_IO, err);
        return DUGKS_OK;
    });
}

int dugks_destroy(dugks_handle* h) {
    delete h;
    return DUGKS_OK;
}

const char* dugks_last_error(const dugks_handle* h) {
    if (!h) return g_err.c_str();
    return h->err.c_str();
}

const char* dugks_global_error(void) { return g_err.c_str(); }

int dugks_get_info(dugks_handle* h, dugks_info* info) {
    if (!info) return DUGKS_ERR_ARG;
    return call(h, [&](dugks::Solver& s) -> int { s.info(*info); return DUGKS_OK; });
}

int dugks_set_dt(dugks_handle* h, double dt) {
    return call(h, [&](dugks::Solver& s) -> int {
        if (!(dt > 0)) return s.fail(DUGKS_ERR_ARG, "dt must be positive");
        s.setDt(dt);
        return DUGKS_OK;
    });
}

int dugks_get_dt(dugks_handle* h, double* dt) {
    if (!dt) return DUGKS_ERR_ARG;
    return call(h, [&](dugks::Solver& s) -> int { *dt = s.dt(); return DUGKS_OK; });
}

int dugks_set_stream(dugks_handle* h, void* stream) {
    return call(h, [&](dugks::Solver& s) -> int { return s.setStream(static_cast<cudaStream_t>(stream)); });
}

int dugks_step(dugks_handle* h, int32_t nsteps) {
    return call(h, [&](dugks::Solver& s) -> int { return s.evolution(nsteps); });
}

int dugks_synchronize(dugks_handle* h) {
    return call(h, [&](dugks::Solver& s) -> int { return s.synchronize(); });
}

int dugks_get_conum(dugks_handle* h, double* max_co, double* mean_co) {
    if (!max_co || !mean_co) return DUGKS_ERR_ARG;
    return call(h, [&](dugks::Solver& s) -> int { return s.getCoNum(*max_co, *mean_co); });
}

int dugks_get_macros(dugks_handle* h, double* rho, double* U, double* T, double* q, double* tau) {
    return call(h, [&](dugks::Solver& s) -> int { return s.macros(rho, U, T, q, tau); });
}

int dugks_get_face_macros(dugks_handle* h, double* rho, double* U, double* T, double* q, double* tau) {
    return call(h, [&](dugks::Solver& s) -> int { return s.faceMacros(rho, U, T, q, tau); });
}

int dugks_get_wall(dugks_handle* h, int32_t patch, double* rho_w, double* q_wall, double* stress_wall) {
    return call(h, [&](dugks::Solver& s) -> int { return s.wall(patch, rho_w, q_wall, stress_wall); });
}

int dugks_get_boundary(dugks_handle* h, int32_t patch, double* rho, double* U, double* T) {
    return call(h, [&](dugks::Solver& s) -> int { return s.boundary(patch, rho, U, T); });
}

int dugks_get_residual(dugks_handle* h, double res[3]) {
    if (!res) return DUGKS_ERR_ARG;
    return call(h, [&](dugks::Solver& s) -> int { return s.residual(res); });
}

int dugks_get_dist(dugks_handle* h, double* g, double* hh) {
    return call(h, [&](dugks::Solver& s) -> int { return s.getDist(g, hh); });
}

int dugks_set_dist(dugks_handle* h, const double* g, const double* hh) {
    return call(h, [&](dugks::Solver& s) -> int { return s.setDist(g, hh); });
}

int dugks_checkpoint_size(dugks_handle* h, size_t* bytes) {
    if (!bytes) return DUGKS_ERR_ARG;
    return call(h, [&](dugks::Solver& s) -> int { *bytes = s.checkpointSize(); return DUGKS_OK; });
}

int dugks_checkpoint_save(dugks_handle* h, void* buf, size_t bytes) {
    if (!buf) return DUGKS_ERR_ARG;
    return call(h, [&](dugks::Solver& s) -> int { return s.checkpointSave(buf, bytes); });
}

int dugks_checkpoint_load(dugks_handle* h, const void* buf, size_t bytes) {
    if (!buf) return DUGKS_ERR_ARG;
    return call(h, [&](dugks::Solver& s) -> int { return s.checkpointLoad(buf, bytes); });
}

int dugks_profile_step(dugks_handle* h, int32_t nsteps, char* names, size_t names_len, double* ms,
                       int32_t max_kernels, int32_t* n_kernels) {
    if (nsteps <= 0 || !ms || !n_kernels) return DUGKS_ERR_ARG;
    return call(h, [&](dugks::Solver& s) -> int {
        std::vector<std::string> nm;
        std::vector<double> t;
        int rc = s.profile(nsteps, nm, t);
        if (rc != DUGKS_OK) return rc;
        *n_kernels = (int32_t)t.size();
        std::string joined;
        for (size_t i = 0; i < t.size(); ++i) {
            if ((int32_t)i < max_kernels) ms[i] = t[i];
            joined += nm[i];
            joined += '\n';
        }
        if (names && names_len) {
            std::strncpy(names, joined.c_str(), names_len - 1);
            names[names_len - 1] = 0;
        }
        return DUGKS_OK;
    });
}

int dugks_macros_noalloc(dugks_handle* h, const double* g, const double* hh, double* rho, double* U, double* T,
                         double* q) {
    return call(h, [&](dugks::Solver& s) -> int {
        std::string err;
        int prev = -1;  // the caller's current device, restored before returning
        if (cudaGetDevice(&prev) != cudaSuccess) {
            cudaGetLastError();
            return s.fail(DUGKS_ERR_CUDA, "dugks_macros_noalloc: cudaGetDevice failed");
        }
        if (prev != s.device()) {
            const cudaError_t e = cudaSetDevice(s.device());
            if (e != cudaSuccess) {
                cudaGetLastError();
                return s.fail(DUGKS_ERR_CUDA, std::string("dugks_macros_noalloc: cudaSetDevice: ") + cudaGetErrorString(e));
            }
        }
        const int rc = dugks::macros_noalloc(s.stepArgs(), s.device(), s.stream(), g, hh, rho, U, T, q, err);
        if (prev != s.device()) cudaSetDevice(prev);
        if (rc != DUGKS_OK) return s.fail(rc, err);
        return DUGKS_OK;
    });
}

int dugks_launches_per_step(dugks_handle* h, int32_t* n) {
    if (!n) return DUGKS_ERR_ARG;
    return call(h, [&](dugks::Solver& s) -> int { *n = s.launchesPerStep(); return DUGKS_OK; });
}

}  // extern "C"

namespace {
int to_objective(dugks_handle* h, const dugks_objective* o, dugks::Objective& r) {
    if (!o) return DUGKS_ERR_ARG;
    r.nSteps = o->n_steps;
    r.avgFirst = o->avg_first;
    r.qPatch = o->q_patch;
    r.stressPatch = o->stress_patch;
    r.ckptEvery = o->checkpoint_every;
    const int nP = (int)h->patchKind.size();
    for (int p : {r.qPatch, r.stressPatch})
        if (p < -1 || p >= nP || (p >= 0 && h->patchKind[p] != DUGKS_PATCH_MAXWELL)) return DUGKS_ERR_ARG;
    return DUGKS_OK;
}
}  // namespace

extern "C" {

int dugks_objective_value(dugks_handle* h, const dugks_objective* o, double* J) {
    if (!h || !h->solver || !J) return DUGKS_ERR_ARG;
    dugks::Objective ob;
    if (int e = to_objective(h, o, ob)) { h->err = "objective: bad patch or null descriptor"; return e; }
    return call(h, [&](dugks::Solver& s) -> int { return dugks::objective_value(s, ob, *J); });
}

int dugks_objective_tangent(dugks_handle* h, const dugks_objective* o, const double* dTw, double ds, double* J,
                            double* dJ) {
    if (!h || !h->solver || !J || !dJ) return DUGKS_ERR_ARG;
    dugks::Objective ob;
    if (int e = to_objective(h, o, ob)) { h->err = "objective: bad patch or null descriptor"; return e; }
    return call(h, [&](dugks::Solver& s) -> int { return dugks::objective_tangent(s, ob, dTw, ds, *J, *dJ); });
}

int dugks_objective_adjoint(dugks_handle* h, const dugks_objective* o, double* J, double* dJ_dTw, double* dJ_ds) {
    if (!h || !h->solver || !J || !dJ_ds) return DUGKS_ERR_ARG;
    dugks::Objective ob;
    if (int e = to_objective(h, o, ob)) { h->err = "objective: bad patch or null descriptor"; return e; }
    return call(h, [&](dugks::Solver& s) -> int { return dugks::objective_adjoint(s, ob, *J, dJ_dTw, *dJ_ds); });
}

}  // extern "C"

struct dugks_batch {
    std::unique_ptr<dugks::Batch> b;
};

namespace {
template <typename F>
int bcall(dugks_batch* h, F&& f) {
    if (!h || !h->b) return DUGKS_ERR_ARG;
    try {
        return f(*h->b);
    } catch (const std::exception& e) {
        h->b->fail(DUGKS_ERR_ARG, e.what());
        return DUGKS_ERR_ARG;
    }
}
}  // namespace

extern "C" {

int dugks_batch_create(const dugks_case_desc* descs, int32_t n_cases, int32_t autotune, dugks_batch** out) {
    if (!descs || !out || n_cases < 1) { g_err = "batch: null argument or no cases"; return DUGKS_ERR_ARG; }
    *out = nullptr;
    try {
        std::string err;
        int code = DUGKS_OK;
        auto b = dugks::Batch::create(descs, n_cases, autotune, err, code);
        if (!b) { g_err = err; return code; }
        *out = new dugks_batch{std::move(b)};
        return DUGKS_OK;
    } catch (const std::exception& e) {
        g_err = e.what();
        return DUGKS_ERR_ARG;
    }
}

int dugks_batch_destroy(dugks_batch* b) {
    delete b;
    return DUGKS_OK;
}

const char* dugks_batch_last_error(const dugks_batch* b) {
    if (!b || !b->b) return g_err.c_str();
    return b->b->error().c_str();
}

int dugks_batch_set_dt(dugks_batch* b, int32_t i, double dt) {
    return bcall(b, [&](dugks::Batch& x) { return x.setDt(i, dt); });
}

int dugks_batch_step(dugks_batch* b, int32_t nsteps) {
    return bcall(b, [&](dugks::Batch& x) { return x.step(nsteps); });
}

int dugks_batch_synchronize(dugks_batch* b) {
    return bcall(b, [&](dugks::Batch& x) { return x.synchronize(); });
}

int dugks_batch_get_macros(dugks_batch* b, int32_t i, double* rho, double* U, double* T, double* q) {
    return bcall(b, [&](dugks::Batch& x) {
        if (i < 0 || i >= x.nCases()) return x.fail(DUGKS_ERR_ARG, "case index out of range");
        if (int e = x.synchronize()) return e;
        if (int e = x.at(i).macros(rho, U, T, q, nullptr)) return x.fail(e, x.at(i).error());
        return (int)DUGKS_OK;
    });
}

int dugks_batch_get_info(dugks_batch* b, dugks_batch_info* out) {
    if (!out) return DUGKS_ERR_ARG;
    return bcall(b, [&](dugks::Batch& x) {
        x.info(*out);
        return (int)DUGKS_OK;
    });
}

int dugks_batch_set_wait_limit(dugks_batch* b, int64_t polls) {
    if (polls < 0) return DUGKS_ERR_ARG;
    return bcall(b, [&](dugks::Batch& x) -> int {
        x.setWaitLimit(polls);
        return DUGKS_OK;
    });
}

}  // extern "C"

