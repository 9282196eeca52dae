"""CPU tests of the FP64 oracle: two independent restatements agree, results
do not depend on the thread count, and physics invariants hold."""
import numpy as np
import pytest

from conftest import rel_err


def _case2d(n=8, nxi=8, **kw):
    from dugksfoam_gb300 import cases

    return cases.cavity2d(n=n, nxi=nxi, **kw)


@pytest.mark.parametrize("kind", ["quad", "tri", "hex"])
def test_c_oracle_matches_numpy_restatement(oracle_lib, kind):
    from dugksfoam_gb300 import cases
    from oracle.oracle import NumpyOracle, Oracle

    if kind == "quad":
        case = _case2d(9, 8)
    elif kind == "tri":
        case = cases.make_case(cases.delaunay_mesh(200, 10, seed=1), *cases.gas_from_kn(0.05), 8,
                               4.0 * np.sqrt(2 * 208.0 * 273.0))
    else:
        case = cases.cavity3d(n=4, nxi=6)
    dt = cases.stable_dt(case)
    a, b = Oracle(case), NumpyOracle(case)
    a.step(dt, 15)
    b.step(dt, 15)
    ca, cb = a.cell(), b.cell()
    for k in ("rho", "U", "T", "q"):
        einf, el2 = rel_err(ca[k], cb[k])
        assert einf < 1e-12 and el2 < 1e-12, (kind, k, einf)


def test_oracle_thread_count_bit_identical(oracle_lib):
    from dugksfoam_gb300 import cases
    from oracle.oracle import Oracle

    case = _case2d(10, 8)
    dt = cases.stable_dt(case)
    out = []
    for th in (1, 3):
        o = Oracle(case, threads=th)
        o.step(dt, 5)
        out.append(o.cell())
    for k in ("rho", "U", "T", "q"):
        assert np.array_equal(out[0][k], out[1][k]), k


def test_mirror_symmetry_of_reflected_lid(oracle_lib):
    """Lid moving -x on the x-mirrored cavity gives the mirrored flow."""
    from dugksfoam_gb300 import cases
    from oracle.oracle import Oracle

    n = 8
    a = _case2d(n, 8, lid_u=50.0)
    b = _case2d(n, 8, lid_u=-50.0)
    dt = cases.stable_dt(a)
    oa, ob = Oracle(a), Oracle(b)
    oa.step(dt, 30)
    ob.step(dt, 30)
    ca, cb = oa.cell(), ob.cell()
    idx = np.arange(n * n).reshape(n, n)  # [j][i]
    mir = idx[:, ::-1].ravel()
    assert np.abs(ca["rho"] - cb["rho"][mir]).max() <= 1e-12 * ca["rho"].max()
    assert np.abs(ca["T"] - cb["T"][mir]).max() <= 1e-12 * ca["T"].max()
    assert np.abs(ca["U"][:, 0] + cb["U"][mir, 0]).max() <= 1e-10 * np.abs(ca["U"]).max()
    assert np.abs(ca["U"][:, 1] - cb["U"][mir, 1]).max() <= 1e-10 * np.abs(ca["U"]).max()


def test_rest_state_stays_near_rest(oracle_lib):
    """No lid and isothermal walls: the gas stays at rest to quadrature accuracy."""
    from dugksfoam_gb300 import cases
    from oracle.oracle import Oracle

    case = _case2d(8, 12, lid_u=0.0)  # 12 nodes -> trapezoid rule (spectral for Gaussians)
    o = Oracle(case)
    o.step(cases.stable_dt(case), 20)
    c = o.cell()
    assert np.abs(c["U"]).max() < 1e-3
    assert np.abs(c["T"] / 273.0 - 1).max() < 1e-4


def test_geometry_against_numpy(oracle_lib):
    from dugksfoam_gb300 import cases, geometry
    from oracle.oracle import Oracle

    case = cases.make_case(cases.delaunay_mesh(150, 8, seed=2), *cases.gas_from_kn(0.05), 6, 1000.0)
    o = Oracle(case)
    g = o.geometry()
    C, V = geometry.cell_centres_volumes(case["mesh"])
    assert np.abs(g["C"] - C).max() < 1e-14
    assert np.abs(g["V"] / V - 1).max() < 1e-12
    assert abs(V.sum() - 1.0 / 8) < 1e-12  # unit square x dz (= 1/n_side)
    assert o.D == 2


def test_initial_state_is_discrete_equilibrium(oracle_lib):
    from oracle.oracle import Oracle

    case = _case2d(4, 28)
    o = Oracle(case)
    g, h = o.dist()
    xi, w = o.dv()
    rho = (w[:, None] * g).sum(0)
    assert np.abs(rho / case["rho0"] - 1).max() < 5e-6  # 28-node Simpson-3/8 quadrature error
