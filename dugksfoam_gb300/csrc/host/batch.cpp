// Batched stepping of independent cases (see batch.h).
#include "batch.h"

#include <algorithm>
#include <cstring>

namespace dugks {

Batch::~Batch() { release(); }

void Batch::release() {
    for (auto& g : graph_)
        if (g) { cudaGraphExecDestroy(g); g = nullptr; }
    for (auto& g : single_)
        if (g) { cudaGraphExecDestroy(g); g = nullptr; }
    bar_ = nullptr;
    tstatus_ = nullptr;  // freed with dev_
    for (auto e : ev_) cudaEventDestroy(e);
    ev_.clear();
    for (auto st : side_) cudaStreamDestroy(st);
    side_.clear();
    for (void* p : dev_) cudaFree(p);
    dev_.clear();
    cases_.clear();
    if (stream_) { cudaStreamDestroy(stream_); stream_ = nullptr; }
}

int Batch::check(cudaError_t e, const char* what) {
    if (e == cudaSuccess) return DUGKS_OK;
    cudaGetLastError();
    return fail(DUGKS_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

int Batch::build(const dugks_case_desc* descs, int n, int npl, int tileCap, int groups) {
    release();
    npl_ = npl;
    tileCap_ = tileCap;
    perCase_ = groups == 0;  // every case its own graph branch with its own kernels
    persistent_ = groups < 0;  // one cooperative launch for all passes and steps
    groups_ = perCase_ ? n : (persistent_ ? 1 : std::max(1, std::min(groups, n)));
    if (int e = check(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking), "stream")) return e;
    for (int g = 1; g < groups_; ++g) {
        cudaStream_t st = nullptr;
        if (int e = check(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking), "stream")) return e;
        side_.push_back(st);
    }
    for (int g = 0; g < 2 * groups_; ++g) {
        cudaEvent_t e = nullptr;
        if (int r = check(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "event")) return r;
        ev_.push_back(e);
    }
    // per-case mode: each case keeps the plan it has when run alone (the
    // same tiles, so bit-identical results)
    fused_set_tuning(npl, tileCap, perCase_);
    cells_ = cellDV_ = 0;
    open_ = false;
    for (int i = 0; i < n; ++i) {
        dugks_case_desc d = descs[i];
        d.precision = DUGKS_FP32_FP64MOM;
        d.pipeline = DUGKS_PIPE_FUSED;
        std::string err;
        int code = DUGKS_OK;
        auto s = Solver::create(d, err, code);
        if (!s) {
            fused_set_tuning(0, 0);
            return fail(code, "case " + std::to_string(i) + ": " + err);
        }
        FusedPipeline* fp = s->fusedPipeline();
        if (!fp || !fp->batchable()) { fused_set_tuning(0, 0); return fail(DUGKS_ERR_UNSUPPORTED, "case is not batchable"); }
        if (!fp->batchKernels()) open_ = true;
        if (s->stepArgs().D != 2) { fused_set_tuning(0, 0); return fail(DUGKS_ERR_UNSUPPORTED, "batched cases must be 2D"); }
        if (int e = s->setStream(stream_)) { fused_set_tuning(0, 0); return fail(e, s->error()); }
        cells_ += s->stepArgs().nC;
        cellDV_ += (long long)s->stepArgs().nC * s->stepArgs().nV;
        cases_.push_back(std::move(s));
    }
    fused_set_tuning(0, 0);
    // open boundary types run each case's own kernels (its graph branch): the
    // batched kernels and the persistent kernel take diffuse walls only
    if (open_ && !perCase_)
        return fail(DUGKS_ERR_UNSUPPORTED, "batch: boundary types other than diffuse walls need the per-case mode");
    const StepArgs a0 = cases_[0]->stepArgs();
    for (auto& c : cases_)
        if (!perCase_ && c->stepArgs().hasH != a0.hasH) return fail(DUGKS_ERR_UNSUPPORTED, "batched cases must agree on h");
    sms_ = cases_[0]->sms();
    dirty_ = true;
    parity_ = 0;
    return DUGKS_OK;
}

int Batch::prepare() {
    for (auto& g : graph_)
        if (g) { cudaGraphExecDestroy(g); g = nullptr; }
    for (auto& g : single_)
        if (g) { cudaGraphExecDestroy(g); g = nullptr; }
    const int n = (int)cases_.size();
    const size_t ab = cases_[0]->fusedPipeline()->batchArgsBytes();
    // groups of about equal work (cells x DVs), largest cases first
    std::vector<int> order(n), group(n, 0);
    for (int i = 0; i < n; ++i) order[i] = i;
    auto work = [&](int i) { return (double)cases_[i]->stepArgs().nC * cases_[i]->stepArgs().Vp; };
    std::sort(order.begin(), order.end(), [&](int x, int y) { return work(x) > work(y); });
    std::vector<double> load(groups_, 0.0);
    for (int i : order) {
        const int g = (int)(std::min_element(load.begin(), load.end()) - load.begin());
        group[i] = g;
        load[g] += work(i);
    }
    const StepArgs a0 = cases_[0]->stepArgs();
    base_.clear();
    for (int i = 0; i < n; ++i) base_.push_back(cases_[i]->stepArgs());
    if (perCase_) {
        for (int q = 0; q < 2; ++q) {
            if (int e = capture(q, 2, graph_[q])) return e;
            if (int e = capture(q, 1, single_[q])) return e;
        }
        dirty_ = false;
        parity_ = 0;
        return DUGKS_OK;
    }
    for (int p = 0; p < 2; ++p) L_[p].assign(groups_, BatchLaunch());
    auto up = [&](const void* src, size_t bytes) -> void* {
        void* ptr = nullptr;
        if (cudaMalloc(&ptr, std::max<size_t>(bytes, 1)) != cudaSuccess) { cudaGetLastError(); return nullptr; }
        dev_.push_back(ptr);
        cudaMemcpy(ptr, src, bytes, cudaMemcpyHostToDevice);
        return ptr;
    };
    for (int g = 0; g < groups_; ++g) {
        std::vector<int> members;
        for (int i = 0; i < n; ++i)
            if (group[i] == g) members.push_back(i);
        const int m = (int)members.size();
        std::vector<unsigned char> host[2] = {std::vector<unsigned char>(ab * m), std::vector<unsigned char>(ab * m)};
        std::vector<int2> wl;
        std::vector<int> faceOff(m + 1, 0), cellOff(m + 1, 0);
        size_t smem = 0;
        int MF = 0;
        for (int j = 0; j < m; ++j) {
            Solver& sv = *cases_[members[j]];
            FusedPipeline* fp = sv.fusedPipeline();
            const StepArgs a = sv.stepArgs();
            for (int p = 0; p < 2; ++p) fp->batchArgs(a, p, host[p].data() + ab * j);
            for (int t = 0; t < fp->batchTiles(); ++t) wl.push_back(make_int2(j, t));
            faceOff[j + 1] = faceOff[j] + a.nA;
            cellOff[j + 1] = cellOff[j] + a.nC;
            smem = std::max(smem, fp->batchSmemFace());
            MF = std::max(MF, fp->batchGatherMF());
        }
        void* args[2] = {up(host[0].data(), host[0].size()), up(host[1].data(), host[1].size())};
        int2* w = static_cast<int2*>(up(wl.data(), wl.size() * sizeof(int2)));
        int* fo = static_cast<int*>(up(faceOff.data(), faceOff.size() * sizeof(int)));
        int* co = static_cast<int*>(up(cellOff.data(), cellOff.size() * sizeof(int)));
        if (!args[0] || !args[1] || !w || !fo || !co) return fail(DUGKS_ERR_OOM, "batch: device allocation failed");
        for (int p = 0; p < 2; ++p) {
            BatchLaunch& L = L_[p][g];
            L.args = args[p];
            L.work = w;
            L.nWork = (int)wl.size();
            L.faceOff = fo;
            L.cellOff = co;
            L.nCases = m;
            L.nFaces = faceOff[m];
            L.smemFace = smem;
            L.MF = MF;
            L.gatherSmem = fused_gather_smem(8, MF, 32 * npl_, a0.hasH != 0);
            L.D = 2;
            L.H = a0.hasH;
            L.npl = npl_;
            if (!fused_batch_prepare(L, sms_)) return fail(DUGKS_ERR_UNSUPPORTED, "batch: no kernels for this case shape");
            if (persistent_ && !fused_batch_persistent_prepare(L, sms_))
                return fail(DUGKS_ERR_UNSUPPORTED, "batch: the persistent kernel does not fit this case shape");
            // the groups run side by side: share the SMs in the persistent gather grid
            L.gatherBlocks = std::max(1, L.gatherBlocks / groups_);
        }
    }
    if (persistent_) {
        const unsigned zero[2] = {0u, 0u};
        const int z = 0;
        bar_ = static_cast<unsigned*>(up(zero, sizeof(zero)));
        tstatus_ = static_cast<int*>(up(&z, sizeof(z)));
        if (!bar_ || !tstatus_) return fail(DUGKS_ERR_OOM, "batch: device allocation failed");
        dirty_ = false;
        parity_ = 0;
        return DUGKS_OK;
    }
    for (int q = 0; q < 2; ++q) {
        if (int e = capture(q, 2, graph_[q])) return e;
        if (int e = capture(q, 1, single_[q])) return e;
    }
    dirty_ = false;
    parity_ = 0;
    return DUGKS_OK;
}

// Graph of `steps` steps from parity q: group 0 on the batch stream, the
// other groups forked onto their own streams and joined at the end.
int Batch::capture(int q, int steps, cudaGraphExec_t& out) {
    cudaGraph_t g = nullptr;
    if (int e = check(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal), "graph capture")) return e;
    cudaError_t ce = cudaEventRecord(ev_[0], stream_);
    for (int k = 1; k < groups_ && ce == cudaSuccess; ++k) ce = cudaStreamWaitEvent(side_[k - 1], ev_[0], 0);
    for (int k = 0; k < groups_; ++k) {
        cudaStream_t st = k == 0 ? stream_ : side_[k - 1];
        for (int s2 = 0; s2 < steps; ++s2) {
            if (perCase_)
                cases_[k]->fusedPipeline()->launchParity(base_[k], (q + s2) & 1, sms_, st);
            else
                for (int pass = 0; pass < 3; ++pass) fused_batch_launch(pass, L_[(q + s2) & 1][k], sms_, st);
        }
    }
    for (int k = 1; k < groups_ && ce == cudaSuccess; ++k) {
        ce = cudaEventRecord(ev_[groups_ + k], side_[k - 1]);
        if (ce == cudaSuccess) ce = cudaStreamWaitEvent(stream_, ev_[groups_ + k], 0);
    }
    cudaError_t ce2 = cudaStreamEndCapture(stream_, &g);
    if (ce == cudaSuccess) ce = ce2;
    if (int e = check(ce, "graph capture")) {
        if (g) cudaGraphDestroy(g);
        return e;
    }
    ce = cudaGraphInstantiate(&out, g, 0);
    cudaGraphDestroy(g);
    return check(ce, "graph instantiate");
}

int Batch::step(int n) {
    if (n < 0) return fail(DUGKS_ERR_ARG, "negative step count");
    for (auto& c : cases_)
        if (!(c->dt() > 0)) return fail(DUGKS_ERR_ARG, "set every case's dt before stepping");
    if (dirty_)
        if (int e = prepare()) return e;
    if (persistent_) {
        if (n > 0) {
            if (int e = check(cudaMemsetAsync(bar_, 0, 2 * sizeof(unsigned), stream_), "barrier reset")) return e;
            if (int e = check(fused_batch_persistent_launch(L_[0][0], L_[1][0], n, parity_, bar_, waitLimit_, tstatus_,
                                                           stream_),
                              "persistent launch"))
                return e;
            parity_ ^= n & 1;
        }
        for (auto& c : cases_) c->advanceExternal(n);
        return DUGKS_OK;
    }
    int left = n;
    while (left >= 2) {
        if (int e = check(cudaGraphLaunch(graph_[parity_], stream_), "graph launch")) return e;
        left -= 2;
    }
    if (left == 1) {
        if (int e = check(cudaGraphLaunch(single_[parity_], stream_), "graph launch")) return e;
        parity_ ^= 1;
    }
    if (int e = check(cudaGetLastError(), "batch step")) return e;
    for (auto& c : cases_) c->advanceExternal(n);
    return DUGKS_OK;
}

int Batch::synchronize() {
    if (int e = check(cudaStreamSynchronize(stream_), "batch synchronize")) return e;
    if (tstatus_) {
        int st = 0;
        if (int e = check(cudaMemcpy(&st, tstatus_, sizeof(int), cudaMemcpyDeviceToHost), "batch status")) return e;
        if (st != 0) {
            cudaMemset(tstatus_, 0, sizeof(int));
            return fail(DUGKS_ERR_TIMEOUT, "batch: a grid barrier wait of the persistent kernel gave up");
        }
    }
    for (size_t i = 0; i < cases_.size(); ++i)
        if (int e = cases_[i]->synchronize()) return fail(e, "case " + std::to_string(i) + ": " + cases_[i]->error());
    return DUGKS_OK;
}

int Batch::setDt(int i, double dt) {
    if (i < 0 || i >= (int)cases_.size()) return fail(DUGKS_ERR_ARG, "case index out of range");
    if (!(dt > 0)) return fail(DUGKS_ERR_ARG, "dt must be positive");
    cases_[i]->setDt(dt);
    dirty_ = true;  // dt is part of the captured kernel arguments
    return DUGKS_OK;
}

void Batch::info(dugks_batch_info& o) const {
    std::memset(&o, 0, sizeof(o));
    o.n_cases = (int32_t)cases_.size();
    o.dv_per_lane = npl_;
    o.tile_cap = tileCap_;
    o.launches_per_step = persistent_ ? 1 : 3 * groups_;  // kernel nodes per step (persistent: one per step call)
    o.steps_per_graph = persistent_ ? 0 : 2;
    o.groups = perCase_ ? 0 : (persistent_ ? -1 : groups_);
    o.cells = cells_;
    o.cell_dv = cellDV_;
    o.n_tuned = (int32_t)std::min<size_t>(tuneMs_.size(), 8);
    for (int k = 0; k < o.n_tuned; ++k) {
        o.tuned_dv_per_lane[k] = tuneNpl_[k];
        o.tuned_tile_cap[k] = tuneCap_[k];
        o.tuned_ms_per_step[k] = tuneMs_[k];
        o.tuned_groups[k] = tuneGroups_[k];
    }
}

std::unique_ptr<Batch> Batch::create(const dugks_case_desc* descs, int n, int autotune, std::string& err, int& code) {
    std::unique_ptr<Batch> b(new Batch());
    code = DUGKS_OK;
    if (!descs || n < 1) { err = "batch: need at least one case"; code = DUGKS_ERR_ARG; return nullptr; }
    // autotune 2: the persistent kernel, untuned
    int bestNpl = 4, bestCap = 0, bestGroups = autotune == 2 ? -1 : 1;
    if (autotune == 1) {
        // candidates: DVs per lane, cap on cells per tile (0: the largest that
        // fits), concurrent groups
        // (groups 0: every case its own graph branch with its own kernels)
        // (groups -1: the persistent kernel)
        const int cand[][3] = {{4, 0, 1}, {4, 0, 4}, {4, 0, 0}, {4, 32, 1}, {2, 0, 1}, {4, 0, -1}};
        double best = 1e300;
        for (auto& c : cand) {
            if (int e = b->build(descs, n, c[0], c[1], c[2])) {
                if (e == DUGKS_ERR_UNSUPPORTED && b->open_) continue;  // a mode the open boundary types exclude
                err = b->err_;
                code = e;
                return nullptr;
            }
            for (auto& s : b->cases_) s->setDt(1e-30);  // timing only: a vanishing step
            b->dirty_ = true;
            cudaEvent_t e0, e1;
            cudaEventCreate(&e0);
            cudaEventCreate(&e1);
            int rc = b->step(2);
            cudaEventRecord(e0, b->stream_);
            if (!rc) rc = b->step(6);
            cudaEventRecord(e1, b->stream_);
            if (!rc) rc = b->check(cudaEventSynchronize(e1), "autotune");
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
            if (rc == DUGKS_ERR_UNSUPPORTED && c[2] < 0) continue;  // the persistent kernel does not fit
            if (rc) { err = b->err_; code = rc; return nullptr; }
            b->tuneNpl_.push_back(c[0]);
            b->tuneCap_.push_back(c[1]);
            b->tuneGroups_.push_back(b->perCase_ ? 0 : (b->persistent_ ? -1 : b->groups_));
            b->tuneMs_.push_back(ms / 6.0);
            if (ms < best) { best = ms; bestNpl = c[0]; bestCap = c[1]; bestGroups = c[2]; }
        }
    }
    std::vector<double> ms = b->tuneMs_;
    std::vector<int> tn = b->tuneNpl_, tc = b->tuneCap_, tg = b->tuneGroups_;
    int rc = b->build(descs, n, bestNpl, bestCap, bestGroups);
    if (rc == DUGKS_ERR_UNSUPPORTED && b->open_ && autotune == 0) rc = b->build(descs, n, bestNpl, bestCap, 0);
    if (rc) { err = b->err_; code = rc; return nullptr; }
    b->tuneMs_ = ms;
    b->tuneNpl_ = tn;
    b->tuneCap_ = tc;
    b->tuneGroups_ = tg;
    return b;
}

}  // namespace dugks
