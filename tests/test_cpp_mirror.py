"""The header-only C++ mirror of fvDVM (include/dugks/fvdvm.hpp) compiles
against the C ABI and links with the library; without a GPU its constructor
throws dugks::Error with DUGKS_ERR_CUDA (no CPU fallback), and the host-only
case inspection works."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

DRIVER = r"""
#include <cstdio>
#include <cstdlib>
#include "dugks/fvdvm.hpp"

int main(int argc, char** argv) {
    const std::string dir = argv[1];
    const int steps = argc > 2 ? std::atoi(argv[2]) : 0;
    const dugks_case_summary s = dugks::FvDVM::inspect(dir);
    std::printf("cells %d walls %d dv %d\n", s.n_cells, s.n_wall_faces, s.n_xi_per_dim);
    try {
        dugks::FvDVM dvm(dir, DUGKS_FP64);  // fvDVM dvm(rho, U, T, &argc, &argv, args)
        double maxCo = 0, meanCo = 0;
        for (int i = 0; i < steps; ++i) {
            dvm.getCoNum(maxCo, meanCo);
            dvm.evolution();
        }
        const std::vector<double> rho = dvm.rhoVol(), U = dvm.Uvol();
        std::printf("nXi %d R %.17g rho0 %.17g Ux0 %.17g maxCo %.17g\n", dvm.nXi(), dvm.R(), rho[0], U[0], maxCo);
        return 0;
    } catch (const dugks::Error& e) {
        std::printf("error %d %s\n", e.code(), e.what());
        return 3;
    }
}
"""


def build_driver(built_lib, tmp_path):
    src = tmp_path / "driver.cpp"
    src.write_text(DRIVER)
    exe = tmp_path / "driver"
    libdir = os.path.dirname(built_lib)
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe),
                    "-L", libdir, "-ldugks", "-Wl,-rpath," + libdir], check=True)
    return exe


@pytest.mark.skipif(shutil.which("g++") is None, reason="no g++")
def test_cpp_mirror_compiles_and_fails_loudly_without_gpu(built_lib, tmp_path):
    import torch

    from dugksfoam_gb300 import cases, foamio

    exe = build_driver(built_lib, tmp_path)
    case = cases.cavity2d(n=6, nxi=6)
    foamio.write_case(case, tmp_path / "case", delta_t=cases.stable_dt(case))
    r = subprocess.run([str(exe), str(tmp_path / "case")], capture_output=True, text=True)
    assert "cells 36 walls 24 dv 6" in r.stdout
    if not torch.cuda.is_available():
        assert r.returncode == 3 and "error 4" in r.stdout, r.stdout + r.stderr
