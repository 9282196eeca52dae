"""Boundary types other than diffuse walls on the CPU: the oracle's restatement
of zeroGradient, mixed (rho fixedValue), farField, pressureIn / pressureOut
(discreteVelocity.C:530-689, fvDVM.C:730-806) and the two symmetry types
(discreteVelocity.C:733-817), 1D meshes, the case writer and reader for them,
and the reference's own symmetry demo case read in place when the tree is
present."""
import os

import numpy as np
import pytest

from conftest import reference_path

REF_SYM = reference_path("demo", "testSymmetry", "symmetry")


def _cases():
    from dugksfoam_gb300 import cases

    return {
        "channel": cases.channel2d(16, 8, nxi=8),
        "open_box": cases.open_box2d(10, nxi=8),
        "half_plane": cases.half_cavity2d(6, 12, nxi=8),
        "half_mod": cases.half_cavity2d(6, 12, nxi=8, sym="symmetryMod"),
        "open_box_zg": cases.open_box2d(10, nxi=8, zero_gradient_tu=True),
        "channel_zg": cases.channel2d(16, 8, nxi=8, inlet_T_zero_gradient=True),
    }


@pytest.mark.parametrize("name", ["channel", "open_box", "half_plane", "half_mod"])
def test_oracle_runs_every_boundary_type(oracle_lib, name):
    from dugksfoam_gb300 import cases
    from oracle.oracle import Oracle

    case = _cases()[name]
    o = Oracle(case)
    o.step(cases.stable_dt(case), 40)
    c = o.cell()
    assert all(np.isfinite(c[k]).all() for k in ("rho", "U", "T", "q"))
    assert c["rho"].min() > 0 and c["T"].min() > 0


def test_pressure_patches_follow_the_characteristic_update(oracle_lib):
    """After a step: inlet rho_b = p_in / (R T_in); outlet T_b = p_out / (R rho_owner)
    and rho_b = rho_i + (p_out - rho_i R T_i) / a_i^2 with the owner's new macros."""
    from dugksfoam_gb300 import cases
    from oracle.oracle import Oracle

    case = _cases()["channel"]
    o = Oracle(case)
    o.step(cases.stable_dt(case), 30)
    m = case["mesh"]
    nI = len(m["neighbour"])
    b, c = o.boundary(), o.cell()
    R, K = case["gas"]["R"], case["gas"]["KInner"]
    inlet, outlet = (next(p for p in m["patches"] if p["name"] == n) for n in ("inlet", "outlet"))
    si = slice(inlet["startFace"] - nI, inlet["startFace"] - nI + inlet["nFaces"])
    assert np.array_equal(b["rho"][si], inlet["pressure"] / R / b["T"][si])
    so = slice(outlet["startFace"] - nI, outlet["startFace"] - nI + outlet["nFaces"])
    own = np.asarray(m["owner"])[outlet["startFace"]:outlet["startFace"] + outlet["nFaces"]]
    rho_i, T_i = c["rho"][own], c["T"][own]
    a2 = R * T_i * (K + 5) / (K + 3)
    np.testing.assert_allclose(b["T"][so], outlet["pressure"] / (R * rho_i), rtol=1e-15)
    np.testing.assert_allclose(b["rho"][so], rho_i + (outlet["pressure"] - rho_i * R * T_i) / a2, rtol=1e-14)
    # the pressure difference drives the gas from the inlet to the outlet
    assert c["U"][:, 0].mean() > 0


@pytest.mark.parametrize("name", ["open_box_zg", "channel_zg"])
def test_zero_gradient_t_and_u_follow_the_owner_cells(oracle_lib, name):
    """Uvol_/Tvol_.correctBoundaryConditions() (fvDVM.C:697-699): after every
    step a zeroGradient T or U patch holds its owner cells' new values; a
    pressureIn patch then sets rho_b = p / (R T_b) from them; and the farField
    or pressureIn inflow differs from the same case with fixed patch values."""
    from dugksfoam_gb300 import cases
    from oracle.oracle import Oracle

    case = _cases()[name]
    dt = cases.stable_dt(case)
    o = Oracle(case)
    o.step(dt, 15)
    m = case["mesh"]
    nI = len(m["neighbour"])
    b, c = o.boundary(), o.cell()
    own = np.asarray(m["owner"])
    for p in m["patches"]:
        sl = slice(p["startFace"] - nI, p["startFace"] - nI + p["nFaces"])
        cells = own[p["startFace"]:p["startFace"] + p["nFaces"]]
        if p.get("T_bc") == "zeroGradient":
            assert np.array_equal(b["T"][sl], c["T"][cells]), p["name"]
            if p.get("bc") == "pressureIn":
                assert np.array_equal(b["rho"][sl], p["pressure"] / case["gas"]["R"] / b["T"][sl])
        if p.get("U_bc") == "zeroGradient":
            assert np.array_equal(b["U"][sl], c["U"][cells]), p["name"]
    fixed = {k: v for k, v in case.items()}
    fixed["mesh"] = dict(m, patches=[{k: v for k, v in p.items() if k not in ("T_bc", "U_bc")} for p in m["patches"]])
    f = Oracle(fixed)
    f.step(dt, 15)
    assert np.abs(f.cell()["T"] - c["T"]).max() > 1e-9 * c["T"].max()


def test_mixed_patch_keeps_its_incoming_maxwellian(oracle_lib):
    """rho fixedValue -> mixed surface patch: the face macros there stay close to
    the patch's Maxwellian half (its incoming DFs are frozen), while a
    zeroGradient face copies its owner cell."""
    from dugksfoam_gb300 import cases
    from oracle.oracle import Oracle

    case = _cases()["open_box"]
    o = Oracle(case)
    o.step(cases.stable_dt(case), 20)
    f = o.face()
    m = case["mesh"]
    top = next(p for p in m["patches"] if p["name"] == "top")
    sl = slice(top["startFace"], top["startFace"] + top["nFaces"])
    # the top patch drives the gas in +x
    assert f["U"][sl, 0].min() > 0


def test_written_cases_read_back(built_lib, tmp_path):
    from dugksfoam_gb300 import foamio, solver

    for name, case in _cases().items():
        d = tmp_path / name
        foamio.write_case(case, d)
        s = solver.inspect_case_dir(d)
        m = case["mesh"]
        assert s["n_cells"] == m["n_cells"] and s["n_patches"] == len(m["patches"])
        walls = sum(p["nFaces"] for p in m["patches"] if solver.patch_bc(p) == "calculatedMaxwell")
        empties = sum(p["nFaces"] for p in m["patches"] if p["type"] == "empty")
        assert s["n_wall_faces"] == walls and s["n_empty_faces"] == empties
        rho, prho = foamio.read_vol_field(d / "0" / "rho")
        for p in m["patches"]:
            assert prho[p["name"]][0] == solver.patch_bc(p)


@pytest.mark.skipif(not REF_SYM or not os.path.isdir(REF_SYM),
                    reason="reference demo case not present (set DUGKS_REFERENCE_ROOT)")
def test_reference_symmetry_demo_case(built_lib):
    """demo/testSymmetry/symmetry: the left half (30 x 60 quads) of the cavity
    with a symmetryMod (DVMsymmetry) patch of 60 faces at x = 0.5."""
    from dugksfoam_gb300 import solver

    s = solver.inspect_case_dir(REF_SYM)
    assert (s["n_cells"], s["n_wall_faces"], s["n_empty_faces"]) == (1800, 120, 3600)
    assert s["n_patches"] == 4


def test_oracle_1d_tube(oracle_lib):
    """A 1D mesh (y and z faces empty: M velocities, fvDVM.C:196-219) between
    two diffuse walls: the expansion runs from the dense half into the thin one."""
    from dugksfoam_gb300 import cases
    from oracle.oracle import Oracle

    case = cases.tube1d(40, nxi=16)
    o = Oracle(case)
    assert o.D == 1 and o.nV == 16
    o.step(cases.stable_dt(case), 100)
    c = o.cell()
    assert np.isfinite(c["q"]).all() and c["T"].min() > 0
    mid = len(c["rho"]) // 2
    assert c["U"][mid - 3:mid + 3, 0].min() > 0.05  # gas moves toward the thin side
    assert c["rho"][:mid].mean() > c["rho"][mid:].mean()


def _box3d():
    """4^3 hexes, 6^3 velocities: farField (x = 0), symmetryPlane (x = 1),
    zeroGradient (z = 1), diffuse walls elsewhere."""
    import math

    from dugksfoam_gb300 import cases

    gas, rho0 = cases.gas_from_kn(0.1)
    mesh = cases.structured_mesh(4, 4, 4, lz=1.0, two_d=False, patch_defs=[
        ("ff", "patch", ["x0"], "farField"), ("sym", "symmetryPlane", ["x1"], "symmetryPlane"),
        ("zg", "patch", ["z1"], "zeroGradient"), ("walls", "wall", ["y0", "y1", "z0"], None)])
    return cases.make_case(mesh, gas, rho0, 6, 4.0 * math.sqrt(2 * gas["R"] * 273.0), two_d=False, lid_u=0.0,
                           bvals={"ff": dict(rho=rho0, T=300.0, U=(30.0, 0.0, 0.0)), "zg": dict(T=273.0)})


@pytest.mark.parametrize("name", ["channel", "open_box", "half_plane", "half_mod", "tube", "box3d", "open_box_zg",
                                  "channel_zg"])
def test_two_independent_restatements_agree(oracle_lib, name):
    """The C oracle and the vectorised numpy restatement (separate code, separate
    summation order) of every boundary type, in 1D, 2D and 3D, agree to ~1e-13."""
    from conftest import rel_err
    from dugksfoam_gb300 import cases
    from oracle.oracle import NumpyOracle, Oracle

    case = {"tube": lambda: cases.tube1d(30, nxi=12), "box3d": _box3d}.get(name, lambda: _cases()[name])()
    dt = cases.stable_dt(case)
    a, b = Oracle(case), NumpyOracle(case)
    a.step(dt, 20)
    b.step(dt, 20)
    ca, cb = a.cell(), b.cell()
    for k in ("rho", "U", "T", "q"):
        einf, el2 = rel_err(cb[k], ca[k])
        assert einf <= 1e-12 and el2 <= 1e-12, (name, k, einf, el2)


def _create_rc(desc):
    import ctypes as C

    from dugksfoam_gb300 import solver

    lib = solver.load_library()
    h = C.c_void_p()
    rc = lib.dugks_create(C.byref(desc), C.byref(h))
    if rc == 0:
        lib.dugks_destroy(h)
    return rc, lib.dugks_global_error().decode()


def test_boundary_descriptions_are_checked_before_device_use(built_lib):
    """Host-side checks of the boundary data, before any device call (so they
    hold without a GPU): pressure patches need patch_pressure, fixedValue and
    farField need positive rho values, and the fused FP64 sweeps refuse open
    types."""
    import numpy as np

    from dugksfoam_gb300 import cases, solver

    d, keep = solver.case_desc(cases.channel2d(8, 4, nxi=8))
    d.patch_pressure = None
    rc, msg = _create_rc(d)
    assert rc == 1 and "patch_pressure" in msg

    box = cases.open_box2d(6, nxi=8)
    box["rhob"] = np.zeros_like(box["rhob"])
    d, keep = solver.case_desc(box)
    rc, msg = _create_rc(d)
    assert rc == 1 and "rho patch values" in msg

    d, keep = solver.case_desc(cases.half_cavity2d(4, 8, nxi=8), precision=solver.FP64,
                               pipeline=solver.PIPE_FUSED)
    rc, msg = _create_rc(d)
    assert rc == 3 and "plain FP64" in msg



def test_channel_reaches_uniform_mass_flux(oracle_lib):
    """Pressure-driven channel (pressureIn / pressureOut, diffuse walls) after
    2000 steps: the mass flux through every cross-section agrees to < 1e-3, so
    the patch updates of fvDVM.C:730-806 drive a steady flow."""
    from dugksfoam_gb300 import cases
    from oracle.oracle import Oracle

    case = cases.channel2d(16, 8, nxi=24)
    o = Oracle(case)
    o.step(cases.stable_dt(case), 2000)
    c = o.cell()
    flux = (c["rho"] * c["U"][:, 0]).reshape(8, 16).mean(0)
    assert flux.min() > 0.1 and (flux.max() - flux.min()) / flux.mean() < 1e-3
