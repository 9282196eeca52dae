"""Case-directory create and time-directory write through the C ABI (GPU).

* dugks_create_from_case_dir on a written case gives bit-identical fields to
  dugks_create on the same in-memory case (17-digit ASCII round trip);
* dugks_write_time writes rho, U, T, q, qSurf, stressSurf that parse back to
  exactly the engine's cell macros and wall outputs, and the written time
  directory is a valid initial-condition directory for the reader.
"""
import shutil

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _case():
    from dugksfoam_gb300 import cases

    return cases.cavity2d(n=10, nxi=8)


@pytest.mark.parametrize("precision", [0, 1])
def test_case_dir_matches_in_memory_create(built_lib, tmp_path, precision):
    from dugksfoam_gb300 import cases, foamio, solver

    case = _case()
    dt = cases.stable_dt(case)
    foamio.write_case(case, tmp_path, delta_t=dt)
    a = solver.FvDVM.from_case_dir(tmp_path, precision=precision)
    b = solver.FvDVM(case, precision=precision)
    assert a.dt == dt
    b.set_dt(dt)
    a.evolution(6)
    b.evolution(6)
    ma, mb = a.macros(), b.macros()
    for k in ("rho", "U", "T", "q"):
        assert np.array_equal(ma[k], mb[k]), k
    a.close()
    b.close()


def test_write_time_round_trip(built_lib, tmp_path):
    from dugksfoam_gb300 import cases, foamio, solver

    case = _case()
    foamio.write_case(case, tmp_path / "case", delta_t=cases.stable_dt(case))
    s = solver.FvDVM.from_case_dir(tmp_path / "case", precision=solver.FP64)
    s.evolution(8)
    s.write(tmp_path / "case", "0.0001")
    m = s.macros()
    d = tmp_path / "case" / "0.0001"
    for k, f in (("rho", "rho"), ("U", "U"), ("T", "T"), ("q", "q")):
        v, _ = foamio.read_vol_field(d / f)
        assert np.array_equal(v, m[k]), k
    rho, prho = foamio.read_vol_field(d / "rho")
    qs, pqs = foamio.read_vol_field(d / "qSurf")
    st, pst = foamio.read_vol_field(d / "stressSurf")
    assert np.all(qs == 0) and np.all(st == 0)
    for p_idx, p in enumerate(case["mesh"]["patches"]):
        if p["type"] != "wall":
            assert prho[p["name"]] == ("empty", None)
            continue
        w = s.wall(p_idx, p["nFaces"])
        assert prho[p["name"]][0] == "calculatedMaxwell"
        assert np.array_equal(prho[p["name"]][1], w["rhoW"])
        assert np.array_equal(pqs[p["name"]][1], w["qWall"])
        assert np.array_equal(pst[p["name"]][1], w["stressWall"])
    # the written directory serves as 0/ of a new case
    shutil.copytree(tmp_path / "case" / "constant", tmp_path / "restart" / "constant")
    shutil.copytree(tmp_path / "case" / "system", tmp_path / "restart" / "system")
    shutil.copytree(d, tmp_path / "restart" / "0")
    r = solver.FvDVM.from_case_dir(tmp_path / "restart", precision=solver.FP64)
    info = r.info()
    assert info["n_cells"] == s.nCells
    r.close()
    s.close()


@pytest.mark.parametrize("precision", [0, 1])
def test_write_df_on_cells(built_lib, tmp_path, precision):
    """fvDVM::writeDFonCells: 0/DF<id> holds g~ of the cell over the velocity
    set, the case's DFwriteCellList by default or an explicit list."""
    import re

    from dugksfoam_gb300 import cases, foamio, solver

    case = _case()
    foamio.write_case(case, tmp_path, delta_t=cases.stable_dt(case), df_cells=[3, 42])
    s = solver.FvDVM.from_case_dir(tmp_path, precision=precision)
    s.evolution(4)
    s.writeDFonCells(tmp_path)
    s.writeDFonCells(tmp_path, cells=[7])
    g, _ = s.dist()

    def read(cid):
        t = (tmp_path / "0" / f"DF{cid}").read_text()
        body = t[t.index("}") + 1:]
        n = int(re.search(r"\b(\d+)\s*\(", body).group(1))
        vals = np.array([float(x) for x in body[body.index("(") + 1:body.rindex(")")].split()])
        assert len(vals) == n == g.shape[1]
        return vals

    for cid in (3, 42, 7):
        assert np.array_equal(read(cid), g[cid]), cid
    s.close()


def test_cpp_mirror_drives_the_engine(built_lib, tmp_path):
    """A dugksFoam-shaped C++ driver over include/dugks/fvdvm.hpp gives the same
    fields as the Python binding on the same case directory."""
    import re
    import subprocess

    from test_cpp_mirror import build_driver

    from dugksfoam_gb300 import cases, foamio, solver

    case = _case()
    foamio.write_case(case, tmp_path / "case", delta_t=cases.stable_dt(case))
    exe = build_driver(built_lib, tmp_path)
    r = subprocess.run([str(exe), str(tmp_path / "case"), "5"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    m = re.search(r"nXi (\d+) R (\S+) rho0 (\S+) Ux0 (\S+)", r.stdout)
    s = solver.FvDVM.from_case_dir(tmp_path / "case", precision=0)
    s.evolution(5)
    mac = s.macros()
    assert int(m.group(1)) == s.nDV and float(m.group(2)) == case["gas"]["R"]
    assert (s.nXi(), s.R(), s.Pr(), s.KInner(), s.nXiPerDim()) == (
        s.nDV, case["gas"]["R"], case["gas"]["Pr"], 0, len(case["xis"]))
    assert float(m.group(3)) == mac["rho"][0] and float(m.group(4)) == mac["U"][0, 0]
    s.close()


def test_zero_gradient_tu_patches_from_case_dir(built_lib, tmp_path):
    """zeroGradient T and U patches in 0/T and 0/U: the case-directory reader
    sets them (the run is bit-identical to the in-memory case that flags them),
    and dugks_write_time writes them back as zeroGradient."""
    from dugksfoam_gb300 import cases, foamio, solver

    case = cases.open_box2d(8, nxi=8, zero_gradient_tu=True)
    dt = cases.stable_dt(case)
    foamio.write_case(case, tmp_path, delta_t=dt)
    a = solver.FvDVM.from_case_dir(tmp_path, precision=solver.FP64)
    b = solver.FvDVM(case, precision=solver.FP64)
    b.set_dt(dt)
    a.evolution(6)
    b.evolution(6)
    ma, mb = a.macros(), b.macros()
    for k in ("rho", "U", "T", "q"):
        assert np.array_equal(ma[k], mb[k]), k
    a.write(tmp_path, "1e-06")
    _, pt = foamio.read_vol_field(tmp_path / "1e-06" / "T")
    _, pu = foamio.read_vol_field(tmp_path / "1e-06" / "U")
    for name in ("farfield", "outflow"):
        assert pt[name][0] == "zeroGradient" and pu[name][0] == "zeroGradient", name
    assert pt["top"][0] == "fixedValue"
    a.close()
    b.close()
