"""The index-checked build (libdugks_checked.so, -DDUGKS_CHECKED=1): every
index the kernels read from mesh or tile data -- tile rows, faces, walls,
stencil entries and cells of the FP32 face sweep, the gather's faces, the
open faces' owners and mirror velocities, the reference pipeline's cell faces
and face cells -- is range-checked on the device; an index out of range would
set the status word to DUGKS_ERR_BOUNDS and be replaced by 0 instead of being
read.  On valid cases of every pipeline and boundary family it reports
nothing and gives the same bits as the normal build."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def checked_lib(built_lib):
    from dugksfoam_gb300 import build

    return build.build(checked=True)


def _cases():
    from dugksfoam_gb300 import cases, solver

    tri = dict(cases.make_case(cases.delaunay_mesh(300, 12, seed=3), *cases.gas_from_kn(0.05), 8,
                               4.0 * np.sqrt(2 * 208.0 * 273.0)), unstructured=True)
    return [
        ("quad12_fp64_ref", cases.cavity2d(n=12, nxi=8), solver.FP64, solver.PIPE_REFERENCE),
        ("tri_fp32", tri, solver.FP32_FP64MOM, solver.PIPE_FUSED),
        ("hex5_fp32", cases.cavity3d(n=5, nxi=6), solver.FP32_FP64MOM, solver.PIPE_FUSED),
        ("open_box_zg_fp64", cases.open_box2d(8, nxi=8, zero_gradient_tu=True), solver.FP64, solver.PIPE_REFERENCE),
        ("open_box_zg_fp32", cases.open_box2d(8, nxi=8, zero_gradient_tu=True), solver.FP32_FP64MOM,
         solver.PIPE_FUSED),
        ("half_plane_fp32", cases.half_cavity2d(6, 12, nxi=8), solver.FP32_FP64MOM, solver.PIPE_FUSED),
    ]


def test_checked_build_is_clean_and_bit_identical(checked_lib):
    from dugksfoam_gb300 import cases, solver

    assert solver.load_library(checked_lib).dugks_checked_build() == 1
    assert solver.load_library().dugks_checked_build() == 0
    for name, case, prec, pipe in _cases():
        out = []
        for path in (None, checked_lib):
            s = solver.FvDVM(case, precision=prec, pipeline=pipe, lib_path=path)
            s.set_dt(cases.case_dt(case))
            s.evolution(12)
            s.synchronize()  # a failed check raises DUGKS_ERR_BOUNDS here
            out.append(s.macros())
            s.close()
        for k in ("rho", "U", "T", "q"):
            assert np.array_equal(out[0][k], out[1][k]), (name, k)
