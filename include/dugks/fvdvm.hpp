// fvdvm.hpp -- header-only C++ mirror of class Foam::fvDVM over the C ABI.
//
// A dugksFoam-shaped driver (src/dugksFoam.C:54-107) keeps its calls:
//   Foam::fvDVM dvm(rho, U, T, &argc, &argv, args);   ->  dugks::FvDVM dvm(caseDir);
//   dvm.getCoNum(maxCo, meanCo);                      ->  the same
//   dvm.evolution();                                  ->  the same
//   dvm.writeDFonCells();                             ->  dvm.writeDFonCells(caseDir)
//   dvm.rhoVol(), Uvol(), Tvol(), qVol(), tauVol()    ->  host copies (vectors)
// Member names follow fvDVM.H:78-377 and the inline accessors of fvDVMI.H.
// Every call that fails throws dugks::Error with the ABI status code.
#pragma once

#include <cstdint>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "dugks/dugks.h"

namespace dugks {

class Error : public std::runtime_error {
public:
    Error(int code, const std::string& what) : std::runtime_error(what), code_(code) {}
    int code() const { return code_; }

private:
    int code_;
};

class FvDVM {
public:
    // fvDVM::fvDVM (fvDVM.C:886-1075) from an OpenFOAM case directory.
    explicit FvDVM(const std::string& caseDir, int precision = DUGKS_FP32_FP64MOM) {
        const int rc = dugks_create_from_case_dir(caseDir.c_str(), precision, &h_);
        if (rc != DUGKS_OK) throw Error(rc, dugks_global_error());
        refresh();
    }
    // ... or from an in-memory case (fvMesh and the 0/ fields filled in by the caller).
    explicit FvDVM(const dugks_case_desc& desc) {
        const int rc = dugks_create(&desc, &h_);
        if (rc != DUGKS_OK) throw Error(rc, dugks_global_error());
        refresh();
    }
    ~FvDVM() {
        if (h_) dugks_destroy(h_);
    }
    FvDVM(const FvDVM&) = delete;
    FvDVM& operator=(const FvDVM&) = delete;
    FvDVM(FvDVM&& o) noexcept : h_(std::exchange(o.h_, nullptr)), info_(o.info_) {}
    FvDVM& operator=(FvDVM&& o) noexcept {
        if (this != &o) {
            if (h_) dugks_destroy(h_);
            h_ = std::exchange(o.h_, nullptr);
            info_ = o.info_;
        }
        return *this;
    }

    // Sizes and parameters of a case directory, on the host only (no GPU).
    static dugks_case_summary inspect(const std::string& caseDir) {
        dugks_case_summary s{};
        const int rc = dugks_inspect_case_dir(caseDir.c_str(), &s);
        if (rc != DUGKS_OK) throw Error(rc, dugks_global_error());
        return s;
    }

    // fvDVM::evolution (fvDVM.C:1086-1108), n steps.
    void evolution(int n = 1) { check(dugks_step(h_, n)); }
    // fvDVM::getCoNum (fvDVM.C:1111-1119).
    void getCoNum(double& maxCo, double& meanCo) { check(dugks_get_conum(h_, &maxCo, &meanCo)); }
    // fvDVM::writeDFonCells (fvDVM.C:877-882): the case's DFwriteCellList, or the given cells.
    void writeDFonCells(const std::string& caseDir, const std::vector<int32_t>* cells = nullptr) {
        check(dugks_write_df_on_cells(h_, caseDir.c_str(), cells ? cells->data() : nullptr,
                                      cells ? (int32_t)cells->size() : 0));
    }
    // runTime.write() of dugksFoam.C:81.
    void write(const std::string& caseDir, const std::string& timeName) {
        check(dugks_write_time(h_, caseDir.c_str(), timeName.c_str()));
    }
    // Time::setDeltaT / deltaTValue.
    void setDeltaT(double dt) { check(dugks_set_dt(h_, dt)); }
    double deltaT() {
        double dt = 0.0;
        check(dugks_get_dt(h_, &dt));
        return dt;
    }
    // Steady-state residuals of dugksFoam.C:88-107: {U, T, rho}.
    void residual(double res[3]) { check(dugks_get_residual(h_, res)); }
    void synchronize() { check(dugks_synchronize(h_)); }

    // rhoVol(), Uvol(), Tvol(), qVol(), tauVol() (fvDVMI.H:42-65): host copies,
    // U and q as [nCells][3].
    std::vector<double> rhoVol() { return cellField(0); }
    std::vector<double> Uvol() { return cellField(1); }
    std::vector<double> Tvol() { return cellField(2); }
    std::vector<double> qVol() { return cellField(3); }
    std::vector<double> tauVol() { return cellField(4); }
    // All cell macros in one call into caller arrays (any may be null).
    void macros(double* rho, double* U, double* T, double* q, double* tau = nullptr) {
        check(dugks_get_macros(h_, rho, U, T, q, tau));
    }
    // rhoSurf(), Usurf(), Tsurf(), qSurf(), tauSurf() (fvDVMI.H:67-95): internal
    // faces followed by the non-empty boundary faces.
    std::vector<double> rhoSurf() { return faceField(0); }
    std::vector<double> Usurf() { return faceField(1); }
    std::vector<double> Tsurf() { return faceField(2); }
    std::vector<double> qSurf() { return faceField(3); }
    std::vector<double> tauSurf() { return faceField(4); }

    // Parameters (fvDVMI.H:97-155).
    int nXi() const { return info_.n_dv; }
    int nXiPerDim() const { return info_.n_xi_per_dim; }
    double xiMax() const { return info_.xi_max; }
    double xiMin() const { return -info_.xi_max; }
    double R() const { return info_.R; }
    double omega() const { return info_.omega; }
    double Tref() const { return info_.Tref; }
    double muRef() const { return info_.muRef; }
    double Pr() const { return info_.Pr; }
    int KInner() const { return info_.KInner; }
    int nCells() const { return info_.n_cells; }
    int nSolutionD() const { return info_.n_solution_d; }

    dugks_handle* handle() { return h_; }

private:
    void check(int rc) {
        if (rc != DUGKS_OK) throw Error(rc, dugks_last_error(h_));
    }
    void refresh() { check(dugks_get_info(h_, &info_)); }
    std::vector<double> cellField(int which) {
        const size_t n = (size_t)info_.n_cells, m = (which == 1 || which == 3) ? 3 : 1;
        std::vector<double> v(n * m);
        double* p[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
        p[which] = v.data();
        check(dugks_get_macros(h_, p[0], p[1], p[2], p[3], p[4]));
        return v;
    }
    std::vector<double> faceField(int which) {
        const size_t n = (size_t)info_.n_internal_faces + info_.n_wall_faces, m = (which == 1 || which == 3) ? 3 : 1;
        std::vector<double> v(n * m);
        double* p[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
        p[which] = v.data();
        check(dugks_get_face_macros(h_, p[0], p[1], p[2], p[3], p[4]));
        return v;
    }

    dugks_handle* h_ = nullptr;
    dugks_info info_{};
};

}  // namespace dugks
