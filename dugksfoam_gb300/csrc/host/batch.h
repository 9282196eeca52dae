// Batched stepping of independent cases (uneven meshes and velocity grids):
// each FP32 pass runs as one launch over every case (tiles, faces and cells of
// all cases in one grid), two steps are captured in a CUDA graph and replayed,
// and an autotuner picks the DVs per lane and the tile-size cap by timing.
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
    int build(const dugks_case_desc* descs, int n, int npl, int tileCap);
    int prepare();  // argument arrays, work lists, graphs
    void release();
    int check(cudaError_t e, const char* what);

    std::vector<std::unique_ptr<Solver>> cases_;
    cudaStream_t stream_ = nullptr;
    int sms_ = 1, npl_ = 4, tileCap_ = 0;
    BatchLaunch L_[2];
    std::vector<void*> dev_;
    cudaGraphExec_t graph_[2] = {nullptr, nullptr};
    int parity_ = 0;
    bool dirty_ = true;
    long long cells_ = 0, cellDV_ = 0;
    std::vector<double> tuneMs_;
    std::vector<int> tuneNpl_, tuneCap_;
    std::string err_;
};

}  // namespace dugks
