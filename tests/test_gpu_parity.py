"""GPU parity: the CUDA engine through the C ABI vs the FP64 CPU oracle.

Tolerances (field-normalised; vector fields by the magnitude of the difference):
  plain FP64 path at the stated step count (61x61 cavity, 2000 steps,
      golden fixture)                  <= 1e-12 (L-inf and L2) on rho, U, T, q
  plain FP64 path, short runs on tiny meshes: <= max(1e-12, 4 x floor), where
      floor is how far an independent FP64 restatement (numpy) sits from the
      oracle on the same run -- early in a transient U and q are near zero in
      most cells and two correct FP64 codes already differ by ~1e-11 in L2
  FP32 bulk / FP64 moments path       <= 1e-5
"""
import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu

FIELDS = ("rho", "U", "T", "q")
TOL64 = 1e-12
TOL32 = 1e-5


def _small_cases():
    from dugksfoam_gb300 import cases

    return {
        "quad12": (cases.cavity2d(n=12, nxi=8), 20),
        "tri": (dict(cases.make_case(cases.delaunay_mesh(300, 12, seed=3), *cases.gas_from_kn(0.05), 8,
                                     4.0 * np.sqrt(2 * 208.0 * 273.0)), unstructured=True), 20),
        "hex5": (cases.cavity3d(n=5, nxi=6), 10),
    }


_FLOOR = {}


def _noise_floor(name):
    """Distance between two independent FP64 restatements (C oracle vs numpy)."""
    from dugksfoam_gb300 import cases
    from oracle.oracle import NumpyOracle, Oracle

    if name not in _FLOOR:
        case, steps = _small_cases()[name]
        dt = cases.case_dt(case)
        a, b = Oracle(case), NumpyOracle(case)
        a.step(dt, steps)
        b.step(dt, steps)
        ca, cb = a.cell(), b.cell()
        _FLOOR[name] = {k: rel_err(cb[k], ca[k]) for k in FIELDS}
    return _FLOOR[name]


def _run_pair(case, steps, precision, pipeline=0):
    from dugksfoam_gb300 import cases, solver
    from oracle.oracle import Oracle

    dt = cases.case_dt(case)
    ref = Oracle(case)
    ref.step(dt, steps)
    s = solver.FvDVM(case, precision=precision, pipeline=pipeline)
    s.set_dt(dt)
    s.evolution(steps)
    return s, ref


@pytest.mark.parametrize("name", ["quad12", "tri", "hex5"])
def test_fp64_reference_pipeline_matches_oracle(built_lib, oracle_lib, name):
    from dugksfoam_gb300 import solver

    case, steps = _small_cases()[name]
    s, ref = _run_pair(case, steps, solver.FP64, solver.PIPE_REFERENCE)
    got, want = s.macros(), ref.cell()
    floor = _noise_floor(name)
    for k in FIELDS:
        einf, el2 = rel_err(got[k], want[k])
        tinf, tl2 = max(TOL64, 4 * floor[k][0]), max(TOL64, 4 * floor[k][1])
        assert einf <= tinf and el2 <= tl2, (name, k, einf, el2, floor[k])
    # face macros and wall state
    fm = s.face_macros()
    of = ref.face()
    nI = len(case["mesh"]["neighbour"])
    wall_faces = [p for p in case["mesh"]["patches"] if p["type"] == "wall"]
    glob = list(range(nI)) + [f for p in wall_faces for f in range(p["startFace"], p["startFace"] + p["nFaces"])]
    for k in ("rho", "T"):
        einf, _ = rel_err(fm[k], of[k][glob])
        assert einf <= TOL64, ("face", k, einf)
    ow = ref.wall()
    for pi, p in enumerate(case["mesh"]["patches"]):
        if p["type"] != "wall":
            continue
        w = s.wall(pi, p["nFaces"])
        sl = slice(p["startFace"] - nI, p["startFace"] - nI + p["nFaces"])
        assert rel_err(w["rhoW"], ow["rhoW"][sl])[0] <= TOL64
        assert rel_err(w["qWall"], ow["qWall"][sl])[0] <= 1e-11
        assert rel_err(w["stressWall"], ow["stressWall"][sl])[0] <= TOL64
    s.close()


def test_fp64_distribution_matches_oracle(built_lib, oracle_lib):
    from dugksfoam_gb300 import solver

    case, _ = _small_cases()["quad12"]
    s, ref = _run_pair(case, 7, solver.FP64, solver.PIPE_REFERENCE)
    g, h = s.dist()
    og, oh = ref.dist()
    assert np.abs(g - og.T).max() / np.abs(og).max() <= TOL64
    assert np.abs(h - oh.T).max() / np.abs(oh).max() <= TOL64


def test_conum_and_residual(built_lib, oracle_lib):
    from dugksfoam_gb300 import cases, solver
    from oracle.oracle import Oracle

    case = cases.cavity2d(n=12, nxi=8)
    dt = cases.stable_dt(case)
    s = solver.FvDVM(case, precision=solver.FP64, pipeline=solver.PIPE_REFERENCE)
    s.set_dt(dt)
    ref = Oracle(case)
    mx, mean = s.getCoNum()
    omx, omean = ref.conum(dt)
    assert abs(mx - omx) <= 1e-13 * omx and abs(mean - omean) <= 1e-13 * omean
    s.evolution(3)
    ref.step(dt, 3)
    mx, mean = s.getCoNum()
    omx, omean = ref.conum(dt)
    assert abs(mx - omx) <= 1e-12 * omx and abs(mean - omean) <= 1e-12 * omean
    r = s.residual()
    m0 = case["U0"], case["T0"], case["rho0"]
    c = ref.cell()
    wantU = np.linalg.norm(c["U"] - m0[0], axis=1).sum() / np.linalg.norm(c["U"], axis=1).sum()
    wantT = np.abs(c["T"] - m0[1]).sum() / c["T"].sum()
    assert abs(r["U"] - wantU) <= 1e-10 * wantU
    assert abs(r["T"] - wantT) <= 1e-10 * wantT
    s.close()


def test_checkpoint_restart_is_exact(built_lib):
    from dugksfoam_gb300 import cases, solver

    case = cases.cavity2d(n=10, nxi=8)
    dt = cases.stable_dt(case)
    a = solver.FvDVM(case, precision=solver.FP64, pipeline=solver.PIPE_REFERENCE)
    a.set_dt(dt)
    a.evolution(5)
    ck = a.checkpoint()
    a.evolution(5)
    want = a.macros()
    b = solver.FvDVM(case, precision=solver.FP64, pipeline=solver.PIPE_REFERENCE)
    b.restore(ck)
    assert b.dt == dt
    b.evolution(5)
    got = b.macros()
    for k in FIELDS:
        assert np.array_equal(got[k], want[k]), k


def test_dist_roundtrip_and_determinism(built_lib):
    from dugksfoam_gb300 import cases, solver

    case = cases.cavity2d(n=8, nxi=8)
    dt = cases.stable_dt(case)
    runs = []
    for _ in range(2):
        s = solver.FvDVM(case, precision=solver.FP64, pipeline=solver.PIPE_REFERENCE)
        s.set_dt(dt)
        s.evolution(4)
        runs.append(s.macros())
        g, h = s.dist()
        s.set_dist(g, h)
        g2, h2 = s.dist()
        assert np.array_equal(g, g2) and np.array_equal(h, h2)
        s.close()
    for k in FIELDS:
        assert np.array_equal(runs[0][k], runs[1][k]), k


def test_nan_state_is_reported(built_lib):
    from dugksfoam_gb300 import cases, solver

    case = cases.cavity2d(n=6, nxi=6)
    s = solver.FvDVM(case, precision=solver.FP64, pipeline=solver.PIPE_REFERENCE)
    s.set_dt(cases.stable_dt(case))
    g, h = s.dist()
    g[3, :] = np.nan
    s.set_dist(g, h)
    s.evolution(1)
    with pytest.raises(solver.DugksError) as ei:
        s.synchronize()
    assert ei.value.code == 5
    s.close()


@pytest.mark.parametrize("name", ["quad12", "tri", "hex5"])
def test_fused_fp64_matches_oracle(built_lib, oracle_lib, name):
    from dugksfoam_gb300 import solver

    case, steps = _small_cases()[name]
    s, ref = _run_pair(case, steps, solver.FP64, solver.PIPE_FUSED)
    got, want = s.macros(), ref.cell()
    floor = _noise_floor(name)
    for k in FIELDS:
        einf, el2 = rel_err(got[k], want[k])
        # one-pass central moments and colour-ordered flux sums: rounding-level
        tinf, tl2 = max(1e-11, 10 * floor[k][0]), max(1e-11, 10 * floor[k][1])
        assert einf <= tinf and el2 <= tl2, (name, k, einf, el2, floor[k])
    s.close()


@pytest.mark.parametrize("name", ["quad12", "tri", "hex5"])
def test_fused_fp32_matches_oracle(built_lib, oracle_lib, name):
    from dugksfoam_gb300 import solver

    case, steps = _small_cases()[name]
    s, ref = _run_pair(case, steps, solver.FP32_FP64MOM, solver.PIPE_FUSED)
    got, want = s.macros(), ref.cell()
    for k in FIELDS:
        einf, el2 = rel_err(got[k], want[k])
        assert einf <= TOL32 and el2 <= TOL32, (name, k, einf, el2)
    s.close()


def _golden(name):
    import os

    return np.load(os.path.join(os.path.dirname(__file__), "golden", name))


@pytest.mark.parametrize("precision,pipeline,tol", [(0, 1, TOL64), (0, 2, 1e-11), (1, 2, TOL32)])
def test_cavity61_2000_steps_against_golden(built_lib, precision, pipeline, tol):
    """The CPU-runnable workload at its stated step count: 61x61 quads,
    28x28 DVs, 2000 steps, against the committed FP64 oracle fields."""
    from dugksfoam_gb300 import cases, solver

    ref = _golden("cavity61_2000.npz")
    case = cases.cavity2d(n=61, nxi=28)
    s = solver.FvDVM(case, precision=precision, pipeline=pipeline)
    s.set_dt(float(ref["dt"]))
    s.evolution(int(ref["steps"]))
    got = s.macros()
    for k in FIELDS:
        einf, el2 = rel_err(got[k], ref[k])
        assert einf <= tol and el2 <= tol, (k, einf, el2)
    s.close()


def test_fp32_delaunay24k_500_steps_against_fp64(built_lib):
    """The headline workload's shape at a quarter of its size (~25k seeded
    Delaunay triangles, 32x32 velocities, Kn 0.01), 500 steps: the FP32 /
    FP64-moment step within 1e-5 (L-inf and L2) of the plain FP64 step, whose
    pipeline the tests above pin to the oracle at 1e-12."""
    from dugksfoam_gb300 import cases, solver

    case = cases.delaunay2d(n_interior=12300, n_side=200)
    dt = cases.case_dt(case)
    out = {}
    for name, prec, pipe in (("fp32", solver.FP32_FP64MOM, solver.PIPE_FUSED),
                             ("fp64", solver.FP64, solver.PIPE_REFERENCE)):
        s = solver.FvDVM(case, precision=prec, pipeline=pipe)
        s.set_dt(dt)
        s.evolution(500)
        out[name] = s.macros()
        s.close()
    for k in FIELDS:
        einf, el2 = rel_err(out["fp32"][k], out["fp64"][k])
        assert einf <= TOL32 and el2 <= TOL32, (k, einf, el2)


@pytest.mark.parametrize("name,env", [
    ("tri", {"DUGKS_TILE_CELLS": "6"}),                           # many tiles: halo rows, one-sided faces
    ("tri", {"DUGKS_TILE_CELLS": "6", "DUGKS_FACE_GRAD": "1"}),  # per-cell gradients, halo rows apart
    ("hex8", {"DUGKS_TILE_CELLS": "10"}),                         # 3D: per-cell gradients, halo rows apart
])
def test_fused_fp32_small_tiles_match_oracle(built_lib, oracle_lib, monkeypatch, name, env):
    """FP32 face sweep on tiles capped far below what shared memory holds, so
    every tile has halo rows and faces across its boundary (and, with
    per-cell gradients, the single-buffered halo rows refilled after the
    gradient pass), against the FP64 oracle."""
    from dugksfoam_gb300 import cases, solver

    for k, v in env.items():
        monkeypatch.setenv(k, v)
    case, steps = _small_cases()[name] if name != "hex8" else (cases.cavity3d(n=8, nxi=6), 10)
    s, ref = _run_pair(case, steps, solver.FP32_FP64MOM, solver.PIPE_FUSED)
    got, want = s.macros(), ref.cell()
    for k in FIELDS:
        einf, el2 = rel_err(got[k], want[k])
        assert einf <= TOL32 and el2 <= TOL32, (name, env, k, einf, el2)
    s.close()
