"""GPU parity of the boundary types other than diffuse walls: the plain FP64
pipeline through the C ABI against the FP64 oracle on pressure-driven channel
flow (pressureIn / pressureOut), an open box (farField, zeroGradient, rho
fixedValue -> mixed, one wall) and the half cavity with a symmetryPlane or a
symmetryMod (DVMsymmetry) patch, on symmetric velocity grids; the open box and
the channel again with zeroGradient T and U patches, whose values follow their
owner cells after every step (fvDVM.C:697-699).

Tolerance: <= 1e-12 field-normalised (L-inf and L2) on rho, U, T, q after 40
steps, and on the face macros and the boundary patch values (patch velocities
normalised by the cell velocity field: the outlet's is still ~1e-4 of it after
40 steps and comes from the cancellation rho_i R T_i - p_out)."""
import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu

TOL64 = 1e-12
STEPS = 40


def _cases():
    from dugksfoam_gb300 import cases

    return {
        "channel": cases.channel2d(24, 12, nxi=12),
        "open_box": cases.open_box2d(14, nxi=12),
        "half_plane": cases.half_cavity2d(8, 16, nxi=12),
        "half_mod": cases.half_cavity2d(8, 16, nxi=12, sym="symmetryMod"),
        # zeroGradient T / U on farField, zeroGradient and pressureIn patches
        "open_box_zg": cases.open_box2d(14, nxi=12, zero_gradient_tu=True),
        "channel_zg": cases.channel2d(24, 12, nxi=12, inlet_T_zero_gradient=True),
    }


@pytest.mark.parametrize("name", ["channel", "open_box", "half_plane", "half_mod", "open_box_zg", "channel_zg"])
def test_fp64_boundary_types_match_oracle(built_lib, oracle_lib, name):
    from dugksfoam_gb300 import cases, solver
    from oracle.oracle import Oracle

    case = _cases()[name]
    dt = cases.stable_dt(case)
    ref = Oracle(case)
    ref.step(dt, STEPS)
    s = solver.FvDVM(case, precision=solver.FP64, pipeline=solver.PIPE_AUTO)
    s.set_dt(dt)
    s.evolution(STEPS)
    got, want = s.macros(), ref.cell()
    for k in ("rho", "U", "T", "q"):
        einf, el2 = rel_err(got[k], want[k])
        assert einf <= TOL64 and el2 <= TOL64, (name, k, einf, el2)
    m = case["mesh"]
    nI = len(m["neighbour"])
    active = [p for p in m["patches"] if p["type"] != "empty"]
    glob = list(range(nI)) + [f for p in active for f in range(p["startFace"], p["startFace"] + p["nFaces"])]
    fm, of = s.face_macros(), ref.face()
    for k in ("rho", "T", "U"):
        einf, _ = rel_err(fm[k], of[k][glob])
        assert einf <= TOL64, (name, "face", k, einf)
    ob = ref.boundary()
    for pi, p in enumerate(m["patches"]):
        if p["type"] == "empty" or solver.patch_bc(p) == "calculatedMaxwell":
            continue
        b = s.boundary(pi, p["nFaces"])
        sl = slice(p["startFace"] - nI, p["startFace"] - nI + p["nFaces"])
        for k in ("rho", "T"):
            assert rel_err(b[k], ob[k][sl])[0] <= TOL64, (name, p["name"], k)
        du = np.linalg.norm(b["U"] - ob["U"][sl], axis=1).max()
        assert du <= TOL64 * np.linalg.norm(want["U"], axis=1).max(), (name, p["name"], "U", du)
    s.close()


@pytest.mark.parametrize("name", ["channel", "open_box", "half_plane", "half_mod", "open_box_zg", "channel_zg"])
def test_fp32_boundary_types_match_oracle(built_lib, oracle_lib, name):
    """FP32 bulk / FP64 moments with zeroGradient, fixedValue, farField, the
    pressure and the symmetry patches: within 1e-5 of the FP64 oracle (the FP32
    path's bound)."""
    from dugksfoam_gb300 import cases, solver
    from oracle.oracle import Oracle

    case = _cases()[name]
    dt = cases.stable_dt(case)
    ref = Oracle(case)
    ref.step(dt, STEPS)
    s = solver.FvDVM(case, precision=solver.FP32_FP64MOM)
    s.set_dt(dt)
    s.evolution(STEPS)
    got, want = s.macros(), ref.cell()
    for k in ("rho", "U", "T", "q"):
        einf, el2 = rel_err(got[k], want[k])
        assert einf <= 1e-5 and el2 <= 1e-5, (name, k, einf, el2)
    s.close()


def test_fused_fp64_sweeps_refuse_open_boundaries(built_lib):
    from dugksfoam_gb300 import solver

    with pytest.raises(solver.DugksError) as e:
        solver.FvDVM(_cases()["half_plane"], precision=solver.FP64, pipeline=solver.PIPE_FUSED)
    assert e.value.code == 3  # DUGKS_ERR_UNSUPPORTED


def test_channel_writes_a_restartable_time_directory(built_lib, tmp_path):
    """dugks_write_time on pressure patches: rho carries its type and pressure
    keyword, U and T the updated patch values; the directory reads back."""
    from dugksfoam_gb300 import cases, foamio, solver

    case = _cases()["channel"]
    foamio.write_case(case, tmp_path)
    s = solver.FvDVM.from_case_dir(tmp_path, precision=solver.FP64)
    s.set_dt(cases.stable_dt(case))
    s.evolution(10)
    s.write(tmp_path, "10")
    rho, prho = foamio.read_vol_field(tmp_path / "10" / "rho")
    assert prho["inlet"][0] == "pressureIn" and prho["outlet"][0] == "pressureOut"
    assert "pressureIn" in (tmp_path / "10" / "rho").read_text()
    m = case["mesh"]
    out = next(i for i, p in enumerate(m["patches"]) if p["name"] == "outlet")
    T, pT = foamio.read_vol_field(tmp_path / "10" / "T")
    assert np.array_equal(pT["outlet"][1], s.boundary(out, m["patches"][out]["nFaces"])["T"])
    s.close()
    # the written time directory is a valid starting point
    import shutil

    shutil.rmtree(tmp_path / "0")
    shutil.copytree(tmp_path / "10", tmp_path / "0")
    info = solver.inspect_case_dir(tmp_path)
    assert info["n_cells"] == m["n_cells"]


def test_fp64_1d_tube_matches_oracle(built_lib, oracle_lib):
    """1D mesh on the plain FP64 pipeline (the fused pipelines refuse it)."""
    from dugksfoam_gb300 import cases, solver
    from oracle.oracle import Oracle

    case = cases.tube1d(60, nxi=16)
    dt = cases.stable_dt(case)
    ref = Oracle(case)
    ref.step(dt, STEPS)
    s = solver.FvDVM(case, precision=solver.FP64)
    assert s.info()["n_solution_d"] == 1
    s.set_dt(dt)
    s.evolution(STEPS)
    got, want = s.macros(), ref.cell()
    for k in ("rho", "U", "T", "q"):
        einf, el2 = rel_err(got[k], want[k])
        assert einf <= TOL64 and el2 <= TOL64, ("1d", k, einf, el2)
    s.close()
    with pytest.raises(solver.DugksError) as e:
        solver.FvDVM(case, precision=solver.FP32_FP64MOM)
    assert e.value.code == 3  # DUGKS_ERR_UNSUPPORTED


@pytest.mark.parametrize("precision", [0, 1])
def test_pressure_case_restarts_exactly(built_lib, precision):
    """The checkpoint carries the pressure patches' rho_b, T_b, U_b: a restored
    handle continues bit for bit (FP64 and FP32 pipelines)."""
    from dugksfoam_gb300 import cases, solver

    case = _cases()["channel"]
    dt = cases.stable_dt(case)
    a = solver.FvDVM(case, precision=precision)
    a.set_dt(dt)
    a.evolution(10)
    ck = a.checkpoint()
    a.evolution(10)
    want = a.macros()
    b = solver.FvDVM(case, precision=precision)
    b.restore(ck)
    b.evolution(10)
    got = b.macros()
    for k in ("rho", "U", "T", "q"):
        assert np.array_equal(got[k], want[k]), k
    a.close()
    b.close()
