// Batched stepping of independent cases (uneven meshes and velocity grids):
// the cases are split into G groups of about equal work; each FP32 pass runs
// as one launch over every case of a group (tiles, faces and cells of all its
// cases in one grid); the groups' launch chains are independent branches of
// one CUDA graph (two steps per graph, replayed), so one group's face sweep
// overlaps another's cell gather; an autotuner picks the DVs per lane, the
// tile-size cap and G by timing, or every case as its own branch with its own
// kernels (G = 0), or the persistent kernel (G = -1): every pass of every
// step of every case in one cooperative launch with bounded grid barriers.
#pragma once

#include <memory>
#include <string>
#include <vector>

#include "../cuda/fused.h"
#include "dugks/dugks.h"
#include "solver.h"

namespace dugks {

class Batch {
public:
    static std::unique_ptr<Batch> create(const dugks_case_desc* descs, int n, int autotune, std::string& err,
                                         int& code);
    ~Batch();

    int step(int n);
    int synchronize();
    int setDt(int i, double dt);
    // polls a grid-barrier wait of the persistent kernel makes before it gives up
    void setWaitLimit(long long polls) { waitLimit_ = polls; }
    Solver& at(int i) { return *cases_[i]; }
    int nCases() const { return (int)cases_.size(); }
    void info(dugks_batch_info& out) const;
    const std::string& error() const { return err_; }
    int fail(int code, const std::string& msg) {
        err_ = msg;
        return code;
    }

private:
    Batch() = default;
    int build(const dugks_case_desc* descs, int n, int npl, int tileCap, int groups);
    int prepare();  // argument arrays, work lists, graphs
    void release();
    int check(cudaError_t e, const char* what);

    std::vector<std::unique_ptr<Solver>> cases_;
    cudaStream_t stream_ = nullptr;
    std::vector<cudaStream_t> side_;   // one per group beyond the first (graph capture fork)
    std::vector<cudaEvent_t> ev_;
    int sms_ = 1, npl_ = 4, tileCap_ = 0, groups_ = 1;
    bool perCase_ = false;
    bool persistent_ = false;
    bool open_ = false;         // some case has boundary types other than diffuse walls
    unsigned* bar_ = nullptr;   // persistent kernel: barrier counters
    int* tstatus_ = nullptr;    // persistent kernel: DUGKS_ERR_TIMEOUT when a barrier wait gave up
    long long waitLimit_ = 1LL << 24;
    std::vector<StepArgs> base_;       // base step arguments of each case at graph build
    std::vector<BatchLaunch> L_[2];    // per parity, per group
    std::vector<void*> dev_;
    cudaGraphExec_t graph_[2] = {nullptr, nullptr};   // two steps from parity q
    cudaGraphExec_t single_[2] = {nullptr, nullptr};  // one step from parity q
    int capture(int q, int steps, cudaGraphExec_t& out);
    int parity_ = 0;
    bool dirty_ = true;
    long long cells_ = 0, cellDV_ = 0;
    std::vector<double> tuneMs_;
    std::vector<int> tuneNpl_, tuneCap_, tuneGroups_;
    std::string err_;
};

}  // namespace dugks
