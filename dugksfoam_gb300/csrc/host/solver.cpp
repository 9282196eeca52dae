// dugks::Solver implementation: case set-up, device state, step dispatch.
#include "solver.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "../cuda/fused.h"

namespace dugks {

namespace {
constexpr double kPiHost = 3.14159265358979323846;

struct CkptHeader {
    char magic[8];
    int32_t abi, precision, nC, nV, Vp, nW, hasH, pad;
    double dt;
    int64_t steps;
};
}  // namespace

template <typename T>
T* Solver::dalloc(size_t n) {
    void* p = nullptr;
    size_t bytes = std::max<size_t>(n, 1) * sizeof(T);
    if (cudaMalloc(&p, bytes) != cudaSuccess) {
        cudaGetLastError();
        oom_ = true;
        return nullptr;
    }
    cudaMemset(p, 0, bytes);
    allocs_.push_back(p);
    bytes_ += bytes;
    return static_cast<T*>(p);
}

int Solver::fail(int code, const std::string& msg) {
    err_ = msg;
    return code;
}

int Solver::checkCuda(cudaError_t e, const char* what) {
    if (e == cudaSuccess) return DUGKS_OK;
    cudaGetLastError();
    return fail(DUGKS_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

Solver::~Solver() {
    if (device_ >= 0) cudaSetDevice(device_);
    if (stream_) cudaStreamSynchronize(stream_);
    fused_.reset();
    for (void* p : allocs_) cudaFree(p);
    if (ownStream_) cudaStreamDestroy(ownStream_);
    if (pin_) cudaFreeHost(pin_);
}

std::unique_ptr<Solver> Solver::create(const dugks_case_desc& d, std::string& err, int& code) {
    std::unique_ptr<Solver> s(new Solver());
    code = s->init(d);
    if (code != DUGKS_OK) {
        err = s->err_;
        return nullptr;
    }
    return s;
}

int Solver::init(const dugks_case_desc& d) {
    if (d.precision != DUGKS_FP64 && d.precision != DUGKS_FP32_FP64MOM)
        return fail(DUGKS_ERR_ARG, "precision must be DUGKS_FP64 or DUGKS_FP32_FP64MOM");
    if (d.n_xi_per_dim < 2 || !d.xis || !d.weights) return fail(DUGKS_ERR_ARG, "missing discrete-velocity grid");
    if (!d.rho0 || !d.U0 || !d.T0) return fail(DUGKS_ERR_ARG, "missing initial fields");
    if (!(d.R > 0) || !(d.Tref > 0) || !(d.muRef > 0) || !(d.Pr > 0)) return fail(DUGKS_ERR_ARG, "invalid gas properties");
    precision_ = d.precision;
    pipeline_ = d.pipeline;
    if (pipeline_ == DUGKS_PIPE_AUTO) pipeline_ = precision_ == DUGKS_FP64 ? DUGKS_PIPE_REFERENCE : DUGKS_PIPE_FUSED;
    if (pipeline_ != DUGKS_PIPE_REFERENCE && pipeline_ != DUGKS_PIPE_FUSED) return fail(DUGKS_ERR_ARG, "unknown pipeline");
    if (precision_ == DUGKS_FP32_FP64MOM && pipeline_ == DUGKS_PIPE_REFERENCE)
        return fail(DUGKS_ERR_UNSUPPORTED, "the reference pipeline is FP64 only");

    MeshInput mi;
    mi.nPoints = d.n_points; mi.points = d.points;
    mi.nCells = d.n_cells; mi.nFaces = d.n_faces; mi.nInternal = d.n_internal_faces;
    mi.faceOffsets = d.face_offsets; mi.faceVerts = d.face_verts; mi.owner = d.owner; mi.neighbour = d.neighbour;
    mi.nPatches = d.n_patches; mi.patchStart = d.patch_start; mi.patchSize = d.patch_size; mi.patchKind = d.patch_kind;
    std::string merr;
    if (!build_mesh(mi, mesh_, merr)) return fail(DUGKS_ERR_ARG, merr);
    const Mesh& m = mesh_;
    const int nC = m.nC, nI = m.nI, nW = m.nW, nA = nI + nW, D = m.D;
    if (nW > 0 && (!d.wall_U || !d.wall_T)) return fail(DUGKS_ERR_ARG, "missing wall_U / wall_T");

    // ---- DV set, fvDVM::initialiseDV (fvDVM.C:140-221)
    const int M = d.n_xi_per_dim;
    nXiPerDim_ = M;
    nV_ = D == 3 ? M * M * M : (D == 2 ? M * M : M);
    const int granule = pipeline_ == DUGKS_PIPE_FUSED ? fused_dv_granule(precision_) : 8;
    Vp_ = (nV_ + granule - 1) / granule * granule;
    const int Vp = Vp_;
    std::vector<double> xi(3 * (size_t)Vp, 0.0), w(Vp, 0.0);
    {
        int i = 0;
        if (D == 3) {
            for (int iz = 0; iz < M; ++iz)
                for (int iy = 0; iy < M; ++iy)
                    for (int ix = 0; ix < M; ++ix, ++i) {
                        w[i] = d.weights[iz] * d.weights[iy] * d.weights[ix];
                        xi[i] = d.xis[ix]; xi[Vp + i] = d.xis[iy]; xi[2 * Vp + i] = d.xis[iz];
                    }
        } else if (D == 2) {
            for (int iy = 0; iy < M; ++iy)
                for (int ix = 0; ix < M; ++ix, ++i) {
                    w[i] = d.weights[iy] * d.weights[ix] * 1;
                    xi[i] = d.xis[ix]; xi[Vp + i] = d.xis[iy];
                }
        } else {
            for (int ix = 0; ix < M; ++ix, ++i) {
                w[i] = d.weights[ix] * 1 * 1;
                xi[i] = d.xis[ix];
            }
        }
    }
    xiMax_ = d.xi_max;
    const int K = d.KInner;
    hasH_ = (K + 3 - D) != 0 ? 1 : 0;  // K=0, D=3: h equilibrium is identically 0

    // ---- boundary kinds other than diffuse walls: plain FP64 pipeline only
    int bcMask = 0;
    for (int wf = 0; wf < nW; ++wf) bcMask |= 1 << m.wallKind[wf];
    // the FP32 pipeline takes every type; the fused FP64 sweeps take walls only
    const int fp32Kinds = (1 << DUGKS_PATCH_MAXWELL) | (1 << DUGKS_PATCH_ZERO_GRADIENT) |
                          (1 << DUGKS_PATCH_FIXED_VALUE) | (1 << DUGKS_PATCH_FAR_FIELD) |
                          (1 << DUGKS_PATCH_PRESSURE_IN) | (1 << DUGKS_PATCH_PRESSURE_OUT) |
                          (1 << DUGKS_PATCH_SYMMETRY_MOD) | (1 << DUGKS_PATCH_SYMMETRY_PLANE);
    if (pipeline_ != DUGKS_PIPE_REFERENCE && (bcMask & ~(precision_ == DUGKS_FP32_FP64MOM ? fp32Kinds : 1 << DUGKS_PATCH_MAXWELL)))
        return fail(DUGKS_ERR_UNSUPPORTED, precision_ == DUGKS_FP32_FP64MOM
                                               ? "symmetry patches need the plain FP64 pipeline (DUGKS_FP64)"
                                               : "boundary types other than calculatedMaxwell walls need the plain FP64 "
                                                 "pipeline (DUGKS_PIPE_REFERENCE or DUGKS_PIPE_AUTO)");
    const bool pressureBc = bcMask & ((1 << DUGKS_PATCH_PRESSURE_IN) | (1 << DUGKS_PATCH_PRESSURE_OUT));
    if (pressureBc && !d.patch_pressure) return fail(DUGKS_ERR_ARG, "pressureIn/pressureOut patches need patch_pressure");
    if ((bcMask & ((1 << DUGKS_PATCH_FIXED_VALUE) | (1 << DUGKS_PATCH_FAR_FIELD))) && !d.bnd_rho)
        return fail(DUGKS_ERR_ARG, "fixedValue/farField patches need bnd_rho");

    // ---- boundary data and inComingByRho (fvDVM::setCalculatedMaxwellRhoBC, fvDVM.C:263-309)
    std::vector<double> Uw(3 * (size_t)nW), Tw(nW), incAbs(nW, 1.0), rhoB(nW, 0.0), pB(nW, 0.0), bS0(3 * (size_t)nW);
    std::vector<int> zg(nW, 0);
    int zgMask = 0;
    for (int wf = 0; wf < nW; ++wf) {
        int b = m.wallFace[wf] - nI;
        const int kind = m.wallKind[wf], p = m.wallPatch[wf];
        for (int k = 0; k < 3; ++k) Uw[3 * wf + k] = d.wall_U[3 * b + k];
        for (int k = 0; k < 3; ++k) bS0[3 * wf + k] = m.Sf[3 * (size_t)d.patch_start[p] + k];
        Tw[wf] = d.wall_T[b];
        // zeroGradient T / U: the owner cell's initial value (as OpenFOAM constructs
        // the patch from its field file), updated after every step
        zg[wf] = (d.patch_T_zero_gradient && d.patch_T_zero_gradient[p] ? 1 : 0) |
                 (d.patch_U_zero_gradient && d.patch_U_zero_gradient[p] ? 2 : 0);
        if (zg[wf] && kind == DUGKS_PATCH_MAXWELL)
            return fail(DUGKS_ERR_UNSUPPORTED, "zeroGradient T or U on a diffuse-wall patch is not supported "
                                               "(the wall Maxwellian and inComingByRho are fixed at creation)");
        if (zg[wf] & 1) Tw[wf] = d.T0[m.owner[m.wallFace[wf]]];
        if (zg[wf] & 2)
            for (int k = 0; k < 3; ++k) Uw[3 * wf + k] = d.U0[3 * (size_t)m.owner[m.wallFace[wf]] + k];
        zgMask |= zg[wf];
        if (d.bnd_rho) rhoB[wf] = d.bnd_rho[b];
        if (kind == DUGKS_PATCH_PRESSURE_IN || kind == DUGKS_PATCH_PRESSURE_OUT) {
            // rho_b (and T_b, U_b) from the initial macros: launch_pressure_bc below
            pB[wf] = d.patch_pressure[p];
            if (!(pB[wf] > 0)) return fail(DUGKS_ERR_ARG, "patch pressure must be positive");
        }
        if ((kind == DUGKS_PATCH_FIXED_VALUE || kind == DUGKS_PATCH_FAR_FIELD) && !(rhoB[wf] > 0))
            return fail(DUGKS_ERR_ARG, "fixedValue/farField rho patch values must be positive");
        if (kind != DUGKS_PATCH_MAXWELL) {
            const bool needT = kind == DUGKS_PATCH_FIXED_VALUE || kind == DUGKS_PATCH_FAR_FIELD ||
                               kind == DUGKS_PATCH_PRESSURE_IN || kind == DUGKS_PATCH_PRESSURE_OUT;
            if (needT && !(Tw[wf] > 0)) return fail(DUGKS_ERR_ARG, "boundary temperature must be positive");
            continue;
        }
        if (!(Tw[wf] > 0)) return fail(DUGKS_ERR_ARG, "wall temperature must be positive");
        const double* S = &m.Sf[3 * (size_t)m.wallFace[wf]];
        double acc = 0.0;
        for (int v = 0; v < nV_; ++v) {
            double x0 = xi[v], x1 = xi[Vp + v], x2 = xi[2 * Vp + v];
            double xs = x0 * S[0] + x1 * S[1] + x2 * S[2];
            if (xs < 0) {
                double a0 = Uw[3 * wf] - x0, a1 = Uw[3 * wf + 1] - x1, a2 = Uw[3 * wf + 2] - x2;
                double M0 = 1.0 / std::pow(std::sqrt(2.0 * kPiHost * d.R * Tw[wf]), (double)D) *
                            std::exp(-(a0 * a0 + a1 * a1 + a2 * a2) / (2.0 * d.R * Tw[wf]));
                acc += -w[v] * xs * M0;
            }
        }
        incAbs[wf] = std::fabs(acc);
        if (!(incAbs[wf] > 0)) return fail(DUGKS_ERR_ARG, "wall face with no incoming discrete velocity");
    }
    // ---- symmetry patches: mirror velocity of every velocity, round(|n . (symX, symY, symZ)|)
    // with n the patch's first-face normal (fvDVM.C:140-221, discreteVelocity.C:733-817)
    std::vector<int32_t> symOff(nW, -1), symTab;
    {
        std::vector<int> patchRow(d.n_patches, -1);
        for (int wf = 0; wf < nW; ++wf) {
            const int kind = m.wallKind[wf], p = m.wallPatch[wf];
            if (kind != DUGKS_PATCH_SYMMETRY_MOD && kind != DUGKS_PATCH_SYMMETRY_PLANE) continue;
            if (patchRow[p] < 0) {
                patchRow[p] = (int)(symTab.size() / nV_);
                const double* S0 = &bS0[3 * wf];
                const double mS = std::sqrt(S0[0] * S0[0] + S0[1] * S0[1] + S0[2] * S0[2]);
                const double n[3] = {S0[0] / mS, S0[1] / mS, S0[2] / mS};
                for (int v = 0; v < nV_; ++v) {
                    int ix = v % M, iy = D == 3 ? (v / M) % M : v / M, iz = D == 3 ? v / (M * M) : 0;
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
                        sx = M - ix - 1;
                        sy = 0;
                        sz = 0;
                    }
                    const long t = std::lround(std::fabs(n[0] * sx + n[1] * sy + n[2] * sz));
                    if (t < 0 || t >= nV_)
                        return fail(DUGKS_ERR_UNSUPPORTED, "symmetry patch: mirror velocity index outside the "
                                                           "velocity set (the patch is not normal to a coordinate axis)");
                    symTab.push_back((int32_t)t);
                }
            }
            symOff[wf] = patchRow[p];
        }
    }
    patchFirstWall_.assign(d.n_patches, -1);
    patchNWall_.assign(d.n_patches, 0);
    for (int wf = 0; wf < nW; ++wf) {
        int p = m.wallPatch[wf];
        if (patchFirstWall_[p] < 0) patchFirstWall_[p] = wf;
        patchNWall_[p]++;
    }

    // ---- device
    device_ = d.device;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        device_ = -1;
        return fail(DUGKS_ERR_CUDA, "no CUDA device available");
    }
    if (int e = checkCuda(cudaSetDevice(device_), "cudaSetDevice")) return e;
    cudaDeviceProp prop;
    if (int e = checkCuda(cudaGetDeviceProperties(&prop, device_), "cudaGetDeviceProperties")) return e;
    sms_ = prop.multiProcessorCount;
    if (int e = checkCuda(cudaStreamCreateWithFlags(&ownStream_, cudaStreamNonBlocking), "cudaStreamCreate")) return e;
    stream_ = ownStream_;

    // ---- geometry of active faces
    std::vector<double> Sf(3 * (size_t)nA), dO(3 * (size_t)nA), dN(3 * (size_t)nI);
    std::vector<int32_t> own(nA), nei(nI);
    auto faceOf = [&](int a) { return a < nI ? a : m.wallFace[a - nI]; };
    for (int a = 0; a < nA; ++a) {
        int f = faceOf(a);
        own[a] = m.owner[f];
        for (int k = 0; k < 3; ++k) {
            Sf[3 * a + k] = m.Sf[3 * (size_t)f + k];
            dO[3 * a + k] = m.Cf[3 * (size_t)f + k] - m.C[3 * (size_t)own[a] + k];
        }
        if (a < nI) {
            nei[a] = m.neighbour[f];
            for (int k = 0; k < 3; ++k) dN[3 * a + k] = m.Cf[3 * (size_t)f + k] - m.C[3 * (size_t)nei[a] + k];
        }
    }
    std::vector<int32_t> cellFace(m.cellFace.size());
    for (size_t j = 0; j < cellFace.size(); ++j) cellFace[j] = (m.cellFace[j] << 1) | m.cellSide[j];

    StepArgs& a = base_;
    a.nC = nC; a.nI = nI; a.nW = nW; a.nA = nA; a.nV = nV_; a.Vp = Vp; a.D = D; a.K = K; a.hasH = hasH_;
    a.R = d.R; a.Pr = d.Pr; a.omega = d.omega; a.Tref = d.Tref; a.muRef = d.muRef; a.dt = 0.0;

    auto up = [&](auto* dst, const auto& src) {
        return cudaMemcpy(dst, src.data(), src.size() * sizeof(src[0]), cudaMemcpyHostToDevice);
    };
    double *dSf = dalloc<double>(Sf.size()), *ddO = dalloc<double>(dO.size()), *ddN = dalloc<double>(dN.size());
    int *down = dalloc<int>(nA), *dnei = dalloc<int>(nI);
    double *dpV = dalloc<double>(m.pVec.size()), *dnV = dalloc<double>(m.nVec.size());
    double *dbV = dalloc<double>(m.bVec.size()), *ddcW = dalloc<double>(nW), *dnH = dalloc<double>(m.nHatW.size());
    double* dvol = dalloc<double>(nC);
    int *dcO = dalloc<int>(m.cellOff.size()), *dcF = dalloc<int>(cellFace.size());
    double *dxi = dalloc<double>(xi.size()), *dw = dalloc<double>(w.size());
    double *dUw = dalloc<double>(Uw.size()), *dTw = dalloc<double>(nW), *dinc = dalloc<double>(nW);
    dcI_ = dalloc<double>(nI);
    a.rhoW = dalloc<double>(nW); a.qWall = dalloc<double>(3 * (size_t)nW); a.stressWall = dalloc<double>(9 * (size_t)nW);
    a.rho = dalloc<double>(nC); a.U = dalloc<double>(3 * (size_t)nC); a.T = dalloc<double>(nC);
    a.q = dalloc<double>(3 * (size_t)nC); a.tau = dalloc<double>(nC);
    a.rhoF = dalloc<double>(nA); a.UF = dalloc<double>(3 * (size_t)nA); a.TF = dalloc<double>(nA);
    a.qF = dalloc<double>(3 * (size_t)nA); a.tauF = dalloc<double>(nA);
    a.status = dalloc<int>(1);
    Uo_ = dalloc<double>(3 * (size_t)nC); To_ = dalloc<double>(nC); ro_ = dalloc<double>(nC); red_ = dalloc<double>(8 + 128 * 8);  // results + per-block partials
    if (oom_) return fail(DUGKS_ERR_OOM, "device allocation failed");
    if (cudaHostAlloc(reinterpret_cast<void**>(&pin_), 8 + 8 * sizeof(double), cudaHostAllocDefault) != cudaSuccess) {
        pin_ = nullptr;
        cudaGetLastError();
        return fail(DUGKS_ERR_OOM, "pinned host allocation failed");
    }
    cudaError_t ce = cudaSuccess;
    auto chk = [&](cudaError_t e) { if (ce == cudaSuccess) ce = e; };
    chk(up(dSf, Sf)); chk(up(ddO, dO)); chk(up(ddN, dN)); chk(up(down, own)); chk(up(dnei, nei));
    chk(up(dpV, m.pVec)); chk(up(dnV, m.nVec)); chk(up(dbV, m.bVec)); chk(up(ddcW, m.dcW)); chk(up(dnH, m.nHatW));
    chk(up(dvol, m.V)); chk(up(dcO, m.cellOff)); chk(up(dcF, cellFace)); chk(up(dxi, xi)); chk(up(dw, w));
    chk(up(dUw, Uw)); chk(up(dTw, Tw)); chk(up(dinc, incAbs)); chk(up(dcI_, m.dcI));
    a.Sf = dSf; a.dO = ddO; a.dN = ddN; a.own = down; a.nei = dnei; a.pVec = dpV; a.nVec = dnV; a.bVec = dbV;
    a.dcW = ddcW; a.nHatW = dnH; a.vol = dvol; a.cellOff = dcO; a.cellFace = dcF; a.xi = dxi; a.w = dw;
    a.Uw = dUw; a.Tw = dTw; a.incAbs = dinc;
    a.bcMask = bcMask;
    a.TbM = dTw; a.UbM = dUw;
    {
        int* dk = dalloc<int>(nW);
        double *drB = dalloc<double>(nW), *dpB = dalloc<double>(nW), *dS0 = dalloc<double>(bS0.size());
        int *dsO = dalloc<int>(nW), *dsT = dalloc<int>(std::max<size_t>(symTab.size(), 1));
        int* dzg = dalloc<int>(nW);
        if (oom_) return fail(DUGKS_ERR_OOM, "device allocation failed");
        chk(up(dk, m.wallKind)); chk(up(drB, rhoB)); chk(up(dpB, pB)); chk(up(dS0, bS0)); chk(up(dsO, symOff));
        chk(up(dzg, zg));
        if (!symTab.empty()) chk(up(dsT, symTab));
        a.bKind = dk; a.rhoB = drB; a.pB = dpB; a.bS0 = dS0; a.symOff = dsO; a.symTab = dsT;
        a.bZG = dzg; a.zgMask = zgMask;
    }

    // initial macros; face velocity = linear interpolation (fvDVM.C:1074) for the first CFL
    std::vector<double> UF(3 * (size_t)nA, 0.0), one(nW, 1.0);
    for (int f = 0; f < nI; ++f)
        for (int k = 0; k < 3; ++k)
            UF[3 * f + k] = m.lerpW[f] * d.U0[3 * (size_t)m.owner[f] + k] +
                            (1.0 - m.lerpW[f]) * d.U0[3 * (size_t)m.neighbour[f] + k];
    for (int wf = 0; wf < nW; ++wf)
        for (int k = 0; k < 3; ++k) UF[3 * (nI + wf) + k] = Uw[3 * wf + k];
    for (int c = 0; c < nC; ++c)
        if (!(d.rho0[c] > 0) || !(d.T0[c] > 0)) return fail(DUGKS_ERR_ARG, "initial rho and T must be positive");
    chk(cudaMemcpy(a.rho, d.rho0, nC * sizeof(double), cudaMemcpyHostToDevice));
    chk(cudaMemcpy(a.U, d.U0, 3 * (size_t)nC * sizeof(double), cudaMemcpyHostToDevice));
    chk(cudaMemcpy(a.T, d.T0, nC * sizeof(double), cudaMemcpyHostToDevice));
    chk(cudaMemcpy(Uo_, d.U0, 3 * (size_t)nC * sizeof(double), cudaMemcpyHostToDevice));
    chk(cudaMemcpy(To_, d.T0, nC * sizeof(double), cudaMemcpyHostToDevice));
    chk(cudaMemcpy(ro_, d.rho0, nC * sizeof(double), cudaMemcpyHostToDevice));
    initRho_ = dalloc<double>(nC); initU_ = dalloc<double>(3 * (size_t)nC); initT_ = dalloc<double>(nC);
    if (oom_) return fail(DUGKS_ERR_OOM, "device allocation failed");
    chk(cudaMemcpy(initRho_, d.rho0, nC * sizeof(double), cudaMemcpyHostToDevice));
    chk(cudaMemcpy(initU_, d.U0, 3 * (size_t)nC * sizeof(double), cudaMemcpyHostToDevice));
    chk(cudaMemcpy(initT_, d.T0, nC * sizeof(double), cudaMemcpyHostToDevice));
    chk(up(a.UF, UF));
    chk(up(a.rhoW, one));
    if (ce != cudaSuccess) return checkCuda(ce, "upload");
    // the constructor ends with updatePressureInOutBC on the initial macros
    // (fvDVM.C:1067-1071)
    if (pressureBc) {
        launch_pressure_bc(a, stream_);
        if (int e = checkCuda(cudaStreamSynchronize(stream_), "initial pressure patches")) return e;
    }

    // ---- distributions
    const size_t nCV = (size_t)nC * Vp;
    if (pipeline_ == DUGKS_PIPE_REFERENCE) {
        RefBuffers& b = ref_;
        b.gT = dalloc<double>(nCV); b.gB = dalloc<double>(nCV); b.gG = dalloc<double>(nCV * D);
        b.Gbg = dalloc<double>((size_t)nW * Vp); b.gS = dalloc<double>((size_t)nA * Vp);
        if (hasH_) {
            b.hT = dalloc<double>(nCV); b.hB = dalloc<double>(nCV); b.hG = dalloc<double>(nCV * D);
            b.Gbh = dalloc<double>((size_t)nW * Vp); b.hS = dalloc<double>((size_t)nA * Vp);
        }
        if (bcMask & ((1 << DUGKS_PATCH_SYMMETRY_MOD) | (1 << DUGKS_PATCH_SYMMETRY_PLANE))) {
            b.gSym = dalloc<double>((size_t)nW * Vp);
            if (hasH_) b.hSym = dalloc<double>((size_t)nW * Vp);
        }
        if (oom_) return fail(DUGKS_ERR_OOM, "device allocation failed (distribution buffers)");
        launch_init_state<double>(a, b.gT, b.hT, 1.0, sms_, stream_);
        launch_ref_mixed_init(a, b, stream_);
    } else {
        std::string ferr;
        fused_ = make_fused_pipeline(*this, a, precision_, ferr);
        if (!fused_) return fail(ferr.find("alloc") != std::string::npos ? DUGKS_ERR_OOM : DUGKS_ERR_UNSUPPORTED, ferr);
        gscale_ = fused_->gscale();
        if (std::getenv("DUGKS_VERBOSE")) std::fprintf(stderr, "dugks fused pipeline: %s\n", fused_->describe().c_str());
        fused_->initState(a, sms_, stream_);
    }
    if (int e = checkCuda(cudaGetLastError(), "init kernels")) return e;
    if (int e = checkCuda(cudaStreamSynchronize(stream_), "init sync")) return e;
    return DUGKS_OK;
}

StepArgs Solver::argsNow() const {
    StepArgs a = base_;
    a.dt = dt_;
    return a;
}

int Solver::setStream(cudaStream_t s) {
    cudaSetDevice(device_);
    cudaStreamSynchronize(stream_);
    stream_ = s ? s : ownStream_;
    return DUGKS_OK;
}

int Solver::launchesPerStep() const {
    return pipeline_ == DUGKS_PIPE_REFERENCE ? kRefKernels : fused_->nKernels();
}

int Solver::runStep(bool timed, std::vector<double>* ms, std::vector<cudaEvent_t>* ev) {
    const StepArgs a = argsNow();
    const int nk = launchesPerStep();
    for (int k = 0; k < nk; ++k) {
        if (timed) cudaEventRecord((*ev)[2 * k], stream_);
        if (pipeline_ == DUGKS_PIPE_REFERENCE)
            launch_ref_pass(k, a, ref_, sms_, stream_);
        else
            fused_->launch(k, a, sms_, stream_);
        if (timed) cudaEventRecord((*ev)[2 * k + 1], stream_);
    }
    if (pipeline_ != DUGKS_PIPE_REFERENCE) fused_->endStep(base_);
    (void)ms;
    return checkCuda(cudaGetLastError(), "step launch");
}

int Solver::evolution(int n) {
    if (!(dt_ > 0)) return fail(DUGKS_ERR_ARG, "dt not set (dugks_set_dt)");
    if (n < 0) return fail(DUGKS_ERR_ARG, "negative step count");
    cudaSetDevice(device_);
    for (int s = 0; s < n; ++s) {
        if (int e = runStep(false, nullptr, nullptr)) return e;
        ++steps_;
    }
    return DUGKS_OK;
}

int Solver::synchronize() {
    cudaSetDevice(device_);
    return syncStatus("step");
}

int Solver::syncStatus(const char* what) {
    cudaError_t ce = cudaMemcpyAsync(pinStatus(), base_.status, sizeof(int), cudaMemcpyDeviceToHost, stream_);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(stream_);
    if (int e = checkCuda(ce, what)) return e;
    const int st = *pinStatus();
    if (st != 0) {
        cudaMemset(base_.status, 0, sizeof(int));
        if (st == DUGKS_ERR_BOUNDS)
            return fail(DUGKS_ERR_BOUNDS, "checked build: an index read from mesh or tile data was out of range");
        return fail(st == DUGKS_ERR_TIMEOUT ? DUGKS_ERR_TIMEOUT : DUGKS_ERR_NUMERIC,
                    st == DUGKS_ERR_TIMEOUT ? "device wait timed out"
                                            : "non-finite or non-positive rho/T detected in the cell moments");
    }
    return DUGKS_OK;
}

void Solver::advanceExternal(int n) {
    for (int i = 0; i < n; ++i)
        if (fused_) fused_->endStep(base_);
    steps_ += n;
}

// The Courant number and the cell macros are enqueued behind the step's
// kernels on the engine's stream and finished by one stream wait that also
// reads the status word (an error of the step is reported by these calls).
int Solver::getCoNum(double& maxCo, double& meanCo) {
    cudaSetDevice(device_);
    launch_conum(argsNow(), dcI_, xiMax_, red_, stream_);
    if (int e = checkCuda(cudaMemcpyAsync(pinRed(), red_, 2 * sizeof(double), cudaMemcpyDeviceToHost, stream_), "conum"))
        return e;
    if (int e = syncStatus("conum")) return e;
    maxCo = pinRed()[0] * dt_;
    meanCo = (mesh_.nI > 0 ? pinRed()[1] / mesh_.nI : 0.0) * dt_;
    return DUGKS_OK;
}

int Solver::macros(double* rho, double* U, double* T, double* q, double* tau) {
    cudaSetDevice(device_);
    const size_t n = mesh_.nC;
    cudaError_t ce = cudaSuccess;
    auto cp = [&](double* dst, const double* src, size_t k) {
        if (dst && ce == cudaSuccess) ce = cudaMemcpyAsync(dst, src, k * sizeof(double), cudaMemcpyDeviceToHost, stream_);
    };
    cp(rho, base_.rho, n); cp(U, base_.U, 3 * n); cp(T, base_.T, n); cp(q, base_.q, 3 * n); cp(tau, base_.tau, n);
    if (int e = checkCuda(ce, "get macros")) return e;
    return syncStatus("get macros");
}

int Solver::faceMacros(double* rho, double* U, double* T, double* q, double* tau) {
    if (int e = synchronize()) return e;
    const size_t n = base_.nA;
    cudaError_t ce = cudaSuccess;
    auto cp = [&](double* dst, const double* src, size_t k) {
        if (dst && ce == cudaSuccess) ce = cudaMemcpyAsync(dst, src, k * sizeof(double), cudaMemcpyDeviceToHost, stream_);
    };
    cp(rho, base_.rhoF, n); cp(U, base_.UF, 3 * n); cp(T, base_.TF, n); cp(q, base_.qF, 3 * n); cp(tau, base_.tauF, n);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(stream_);
    return checkCuda(ce, "get face macros");
}

int Solver::wall(int patch, double* rhoW, double* qWall, double* stressWall) {
    if (patch < 0 || patch >= (int)patchFirstWall_.size()) return fail(DUGKS_ERR_ARG, "patch index out of range");
    if (patchNWall_[patch] == 0) return fail(DUGKS_ERR_ARG, "patch has no wall faces");
    if (int e = synchronize()) return e;
    const size_t s = patchFirstWall_[patch], n = patchNWall_[patch];
    cudaError_t ce = cudaSuccess;
    if (rhoW) ce = cudaMemcpy(rhoW, base_.rhoW + s, n * sizeof(double), cudaMemcpyDeviceToHost);
    if (qWall && ce == cudaSuccess) ce = cudaMemcpy(qWall, base_.qWall + 3 * s, 3 * n * sizeof(double), cudaMemcpyDeviceToHost);
    if (stressWall && ce == cudaSuccess)
        ce = cudaMemcpy(stressWall, base_.stressWall + 9 * s, 9 * n * sizeof(double), cudaMemcpyDeviceToHost);
    return checkCuda(ce, "get wall");
}

int Solver::boundary(int patch, double* rho, double* U, double* T) {
    if (patch < 0 || patch >= (int)patchFirstWall_.size()) return fail(DUGKS_ERR_ARG, "patch index out of range");
    if (patchNWall_[patch] == 0) return fail(DUGKS_ERR_ARG, "patch has no active faces");
    if (int e = synchronize()) return e;
    const size_t s = patchFirstWall_[patch], n = patchNWall_[patch];
    const bool wall = mesh_.wallKind[s] == DUGKS_PATCH_MAXWELL;
    cudaError_t ce = cudaSuccess;
    if (rho) ce = cudaMemcpy(rho, (wall ? base_.rhoW : base_.rhoB) + s, n * sizeof(double), cudaMemcpyDeviceToHost);
    if (U && ce == cudaSuccess) ce = cudaMemcpy(U, base_.Uw + 3 * s, 3 * n * sizeof(double), cudaMemcpyDeviceToHost);
    if (T && ce == cudaSuccess) ce = cudaMemcpy(T, base_.Tw + s, n * sizeof(double), cudaMemcpyDeviceToHost);
    return checkCuda(ce, "get boundary");
}

int Solver::residual(double res[3]) {
    cudaSetDevice(device_);
    launch_residual(argsNow(), Uo_, To_, ro_, red_, stream_);
    double* s = pinRed();
    if (int e = checkCuda(cudaMemcpyAsync(s, red_, 6 * sizeof(double), cudaMemcpyDeviceToHost, stream_), "residual"))
        return e;
    if (int e = syncStatus("residual")) return e;
    res[0] = s[1] > 0 ? s[0] / s[1] : 0.0;
    res[1] = s[3] > 0 ? s[2] / s[3] : 0.0;
    res[2] = s[5] > 0 ? s[4] / s[5] : 0.0;
    return DUGKS_OK;
}

int Solver::getDist(double* g, double* h) {
    if (int e = synchronize()) return e;
    const size_t n = (size_t)mesh_.nC * nV_;
    double* tmp = nullptr;
    if (int e = checkCuda(cudaMalloc(&tmp, n * sizeof(double)), "cudaMalloc (export)")) return e;
    cudaError_t ce = cudaSuccess;
    const StepArgs a = argsNow();
    for (int which = 0; which < 2 && ce == cudaSuccess; ++which) {
        double* dst = which == 0 ? g : h;
        if (!dst) continue;
        if (which == 1 && !hasH_) {
            std::fill(h, h + n, 0.0);
            continue;
        }
        if (pipeline_ == DUGKS_PIPE_REFERENCE)
            launch_export_dist<double>(a, which ? ref_.hT : ref_.gT, tmp, 1.0, sms_, stream_);
        else
            fused_->exportDist(a, which, tmp, sms_, stream_);
        ce = cudaMemcpyAsync(dst, tmp, n * sizeof(double), cudaMemcpyDeviceToHost, stream_);
        if (ce == cudaSuccess) ce = cudaStreamSynchronize(stream_);
    }
    cudaFree(tmp);
    return checkCuda(ce, "get dist");
}

int Solver::setDist(const double* g, const double* h) {
    if (int e = synchronize()) return e;
    const size_t n = (size_t)mesh_.nC * nV_;
    double* tmp = nullptr;
    if (int e = checkCuda(cudaMalloc(&tmp, n * sizeof(double)), "cudaMalloc (import)")) return e;
    cudaError_t ce = cudaSuccess;
    const StepArgs a = argsNow();
    for (int which = 0; which < 2 && ce == cudaSuccess; ++which) {
        const double* src = which == 0 ? g : h;
        if (!src || (which == 1 && !hasH_)) continue;
        ce = cudaMemcpyAsync(tmp, src, n * sizeof(double), cudaMemcpyHostToDevice, stream_);
        if (ce != cudaSuccess) break;
        if (pipeline_ == DUGKS_PIPE_REFERENCE)
            launch_import_dist<double>(a, tmp, which ? ref_.hT : ref_.gT, 1.0, sms_, stream_);
        else
            fused_->importDist(a, which, tmp, sms_, stream_);
        ce = cudaStreamSynchronize(stream_);
    }
    cudaFree(tmp);
    return checkCuda(ce, "set dist");
}

// Exact-restart checkpoint layout: header, g~, h~ (storage type), lagged
// boundary gradients, cell macros rho,U,T,q,tau, face velocity, boundary patch
// values rho_b, T_b, U_b (pressure patches change them every step).
size_t Solver::checkpointSize() const {
    const size_t es = precision_ == DUGKS_FP64 ? 8 : 4;
    const size_t nCV = (size_t)mesh_.nC * Vp_, nWV = (size_t)mesh_.nW * Vp_;
    const size_t nd = hasH_ ? 2 : 1;
    return sizeof(CkptHeader) + nd * (nCV + nWV) * es + (size_t)mesh_.nC * 9 * 8 + (size_t)base_.nA * 3 * 8 +
           (size_t)mesh_.nW * 5 * 8;
}

int Solver::checkpointSave(void* buf, size_t n) {
    if (n < checkpointSize()) return fail(DUGKS_ERR_ARG, "checkpoint buffer too small");
    if (int e = synchronize()) return e;
    char* p = static_cast<char*>(buf);
    CkptHeader hd{};
    std::memcpy(hd.magic, "DUGKSCK2", 8);
    hd.abi = DUGKS_ABI_VERSION; hd.precision = precision_; hd.nC = mesh_.nC; hd.nV = nV_; hd.Vp = Vp_;
    hd.nW = mesh_.nW; hd.hasH = hasH_; hd.dt = dt_; hd.steps = steps_;
    std::memcpy(p, &hd, sizeof(hd));
    p += sizeof(hd);
    const size_t es = precision_ == DUGKS_FP64 ? 8 : 4;
    const size_t nCV = (size_t)mesh_.nC * Vp_, nWV = (size_t)mesh_.nW * Vp_;
    cudaError_t ce = cudaSuccess;
    auto get = [&](const void* src, size_t bytes) {
        if (ce == cudaSuccess) ce = cudaMemcpy(p, src, bytes, cudaMemcpyDeviceToHost);
        p += bytes;
    };
    for (int which = 0; which < (hasH_ ? 2 : 1); ++which) {
        const void *T, *G;
        if (pipeline_ == DUGKS_PIPE_REFERENCE) {
            T = which ? ref_.hT : ref_.gT;
            G = which ? ref_.Gbh : ref_.Gbg;
        } else {
            T = fused_->distPtr(which);
            G = fused_->gradBPtr(which);
        }
        get(T, nCV * es);
        get(G, nWV * es);
    }
    const size_t nC = mesh_.nC;
    get(base_.rho, nC * 8); get(base_.U, 3 * nC * 8); get(base_.T, nC * 8); get(base_.q, 3 * nC * 8); get(base_.tau, nC * 8);
    get(base_.UF, (size_t)base_.nA * 3 * 8);
    const size_t nW = mesh_.nW;
    get(base_.rhoB, nW * 8); get(base_.TbM, nW * 8); get(base_.UbM, 3 * nW * 8);
    return checkCuda(ce, "checkpoint save");
}

int Solver::checkpointLoad(const void* buf, size_t n) {
    if (n < sizeof(CkptHeader)) return fail(DUGKS_ERR_ARG, "checkpoint too small");
    const char* p = static_cast<const char*>(buf);
    CkptHeader hd;
    std::memcpy(&hd, p, sizeof(hd));
    if (std::memcmp(hd.magic, "DUGKSCK2", 8) != 0) return fail(DUGKS_ERR_ARG, "not a DUGKS checkpoint (or an older layout)");
    if (hd.precision != precision_ || hd.nC != mesh_.nC || hd.nV != nV_ || hd.Vp != Vp_ || hd.nW != mesh_.nW ||
        hd.hasH != hasH_)
        return fail(DUGKS_ERR_ARG, "checkpoint does not match this case/precision");
    if (n < checkpointSize()) return fail(DUGKS_ERR_ARG, "checkpoint truncated");
    if (int e = synchronize()) return e;
    p += sizeof(hd);
    const size_t es = precision_ == DUGKS_FP64 ? 8 : 4;
    const size_t nCV = (size_t)mesh_.nC * Vp_, nWV = (size_t)mesh_.nW * Vp_;
    cudaError_t ce = cudaSuccess;
    auto put = [&](void* dst, size_t bytes) {
        if (ce == cudaSuccess) ce = cudaMemcpy(dst, p, bytes, cudaMemcpyHostToDevice);
        p += bytes;
    };
    for (int which = 0; which < (hasH_ ? 2 : 1); ++which) {
        void *T, *G;
        if (pipeline_ == DUGKS_PIPE_REFERENCE) {
            T = which ? ref_.hT : ref_.gT;
            G = which ? ref_.Gbh : ref_.Gbg;
        } else {
            T = fused_->distPtr(which);
            G = fused_->gradBPtr(which);
        }
        put(T, nCV * es);
        put(G, nWV * es);
    }
    const size_t nC = mesh_.nC;
    put(base_.rho, nC * 8); put(base_.U, 3 * nC * 8); put(base_.T, nC * 8); put(base_.q, 3 * nC * 8); put(base_.tau, nC * 8);
    put(base_.UF, (size_t)base_.nA * 3 * 8);
    const size_t nW = mesh_.nW;
    put(base_.rhoB, nW * 8); put(base_.TbM, nW * 8); put(base_.UbM, 3 * nW * 8);
    dt_ = hd.dt;
    steps_ = hd.steps;
    if (ce == cudaSuccess && fused_) fused_->refreshDerived(argsNow(), sms_, stream_);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(stream_);
    return checkCuda(ce, "checkpoint load");
}

int Solver::profile(int nsteps, std::vector<std::string>& names, std::vector<double>& ms) {
    if (!(dt_ > 0)) return fail(DUGKS_ERR_ARG, "dt not set (dugks_set_dt)");
    if (int e = synchronize()) return e;
    const int nk = launchesPerStep();
    std::vector<cudaEvent_t> ev(2 * nk);
    for (auto& e : ev) cudaEventCreate(&e);
    ms.assign(nk, 0.0);
    names.clear();
    for (int k = 0; k < nk; ++k)
        names.push_back(pipeline_ == DUGKS_PIPE_REFERENCE ? kRefKernelNames[k] : fused_->kernelName(k));
    int rc = DUGKS_OK;
    for (int s = 0; s < nsteps && rc == DUGKS_OK; ++s) {
        rc = runStep(true, nullptr, &ev);
        ++steps_;
        if (rc == DUGKS_OK) rc = checkCuda(cudaStreamSynchronize(stream_), "profile");
        for (int k = 0; k < nk && rc == DUGKS_OK; ++k) {
            float t = 0.f;
            cudaEventElapsedTime(&t, ev[2 * k], ev[2 * k + 1]);
            ms[k] += t / nsteps;
        }
    }
    for (auto& e : ev) cudaEventDestroy(e);
    return rc;
}

void Solver::info(dugks_info& o) const {
    o.n_cells = mesh_.nC; o.n_faces = mesh_.nF; o.n_internal_faces = mesh_.nI; o.n_wall_faces = mesh_.nW;
    o.n_dv = nV_; o.n_dv_padded = Vp_; o.n_solution_d = mesh_.D; o.has_h = hasH_;
    o.precision = precision_; o.pipeline = pipeline_; o.dt = dt_; o.step_count = steps_;
    o.device_bytes = bytes_ + (fused_ ? fused_->bytes() : 0);
    o.n_xi_per_dim = nXiPerDim_; o.KInner = base_.K;
    o.xi_max = xiMax_; o.R = base_.R; o.omega = base_.omega; o.Tref = base_.Tref; o.muRef = base_.muRef;
    o.Pr = base_.Pr;
}

template double* Solver::dalloc<double>(size_t);
template float* Solver::dalloc<float>(size_t);
template int* Solver::dalloc<int>(size_t);

}  // namespace dugks
