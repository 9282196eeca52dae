"""Batched cases (GPU): uneven meshes and velocity grids advanced together
agree with each case stepped alone with the FP32 pipeline under the same
tuning to FP32 rounding (the batched kernels are separate instantiations of
the same device code, so the compiler may contract multiply-adds differently),
and are bit-reproducible from run to run; the autotuner times its candidates;
an odd step count (one step outside the two-step graph) and a dt change
(graph re-capture) are covered.  The persistent kernel (every pass and step in
one cooperative launch) meets the same bounds, and a grid-barrier wait that
gives up (wait limit 0) is reported as DUGKS_ERR_TIMEOUT with the device still
usable afterwards."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _instances():
    from dugksfoam_gb300 import cases

    return [dict(N=6, M=8, Kn=0.05, lid_u=50.0, Tw=273.0), dict(N=9, M=12, Kn=0.3, lid_u=20.0, Tw=300.0),
            dict(N=7, M=6, Kn=0.01, lid_u=80.0, Tw=260.0)]


def _run_batch(cs, dts):
    from dugksfoam_gb300 import solver

    b = solver.Batch(cs, autotune=False)
    info = b.info()
    assert info["n_cases"] == 3 and info["groups"] == 1 and info["launches_per_step"] == 3
    assert info["dv_per_lane"] == 4
    for i, dt in enumerate(dts):
        b.set_dt(i, dt)
    b.step(7)          # three graph replays and one single step
    b.set_dt(1, 0.9 * dts[1])
    b.step(4)          # re-captured graphs
    out = [b.macros(i) for i in range(len(cs))]
    b.close()
    return out


def test_batch_matches_single_cases_and_oracle(built_lib, oracle_lib):
    from conftest import rel_err
    from dugksfoam_gb300 import cases, solver
    from oracle.oracle import Oracle

    cs = [cases.batch_case(i) for i in _instances()]
    dts = [cases.stable_dt(c) for c in cs]
    got_all = _run_batch(cs, dts)
    again = _run_batch(cs, dts)
    for i in range(len(cs)):
        for k in ("rho", "U", "T", "q"):
            assert np.array_equal(got_all[i][k], again[i][k]), ("reproducible", i, k)
    for i, c in enumerate(cs):
        s = solver.FvDVM(c, precision=solver.FP32_FP64MOM, pipeline=solver.PIPE_FUSED)
        s.set_dt(dts[i])
        s.evolution(7)
        if i == 1:
            s.set_dt(0.9 * dts[1])
        s.evolution(4)
        want, got = s.macros(), got_all[i]
        ref = Oracle(c)
        ref.step(dts[i], 7)
        ref.step(0.9 * dts[1] if i == 1 else dts[i], 4)
        oracle = ref.cell()
        for k in ("rho", "U", "T", "q"):
            for other in (want, oracle):  # the single-case FP32 run and the FP64 oracle
                einf, el2 = rel_err(got[k], other[k])
                assert einf <= 1e-5 and el2 <= 1e-5, (i, k, einf, el2)
        s.close()


def test_batch_autotune(built_lib):
    from dugksfoam_gb300 import cases, solver

    cs = [cases.batch_case(i) for i in _instances()]
    b = solver.Batch(cs, autotune=True)
    info = b.info()
    # five graph candidates and the persistent kernel (groups -1)
    assert len(info["tuned"]) == 6 and all(t["ms_per_step"] > 0 for t in info["tuned"])
    assert info["tuned"][-1]["groups"] == -1
    best = min(info["tuned"], key=lambda t: t["ms_per_step"])
    assert (info["dv_per_lane"], info["tile_cap"], info["groups"]) == (best["dv_per_lane"], best["tile_cap"],
                                                                      best["groups"])
    for i, c in enumerate(cs):
        b.set_dt(i, cases.stable_dt(c))
    b.step(3)
    b.synchronize()
    m = b.macros(2)
    assert np.all(np.isfinite(m["rho"])) and np.all(m["rho"] > 0)
    b.close()


def _run_persistent(cs, dts, wait_limit=None):
    from dugksfoam_gb300 import solver

    b = solver.Batch(cs, persistent=True)
    info = b.info()
    assert info["groups"] == -1 and info["launches_per_step"] == 1
    if wait_limit is not None:
        b.set_wait_limit(wait_limit)
    for i, dt in enumerate(dts):
        b.set_dt(i, dt)
    b.step(7)          # one launch of seven steps
    b.set_dt(1, 0.9 * dts[1])
    b.step(4)
    b.synchronize()
    out = [b.macros(i) for i in range(len(cs))]
    b.close()
    return out


def test_persistent_batch_matches_single_cases_and_oracle(built_lib, oracle_lib):
    from conftest import rel_err
    from dugksfoam_gb300 import cases, solver
    from oracle.oracle import Oracle

    cs = [cases.batch_case(i) for i in _instances()]
    dts = [cases.stable_dt(c) for c in cs]
    got_all = _run_persistent(cs, dts)
    again = _run_persistent(cs, dts)
    for i in range(len(cs)):
        for k in ("rho", "U", "T", "q"):
            assert np.array_equal(got_all[i][k], again[i][k]), ("reproducible", i, k)
    for i, c in enumerate(cs):
        ref = Oracle(c)
        ref.step(dts[i], 7)
        ref.step(0.9 * dts[1] if i == 1 else dts[i], 4)
        oracle = ref.cell()
        for k in ("rho", "U", "T", "q"):
            einf, el2 = rel_err(got_all[i][k], oracle[k])
            assert einf <= 1e-5 and el2 <= 1e-5, (i, k, einf, el2)


def test_persistent_batch_barrier_timeout_is_reported(built_lib):
    """Wait limit 0: the first grid-barrier wait gives up, every block leaves
    the kernel, dugks_batch_synchronize returns DUGKS_ERR_TIMEOUT; a new batch
    then runs normally (the context is intact)."""
    from dugksfoam_gb300 import cases, solver

    cs = [cases.batch_case(i) for i in _instances()]
    dts = [cases.stable_dt(c) for c in cs]
    with pytest.raises(solver.DugksError) as ei:
        _run_persistent(cs, dts, wait_limit=0)
    assert ei.value.code == 6
    out = _run_persistent(cs, dts)
    assert all(np.all(np.isfinite(m["rho"])) and np.all(m["rho"] > 0) for m in out)


def test_batch_with_open_boundary_types(built_lib, oracle_lib):
    """Cases with farField, zeroGradient, fixedValue and pressure patches (and
    zeroGradient U/T) batch in the per-case mode: each case its own kernels as
    a graph branch, bit-identical to the case run alone and within 1e-5 of the
    oracle; the batched and the persistent kernels refuse them."""
    from conftest import rel_err
    from dugksfoam_gb300 import cases, solver
    from oracle.oracle import Oracle

    cs = [cases.open_box2d(8, nxi=8, zero_gradient_tu=True), cases.channel2d(12, 6, nxi=8, inlet_T_zero_gradient=True),
          cases.batch_case(_instances()[0])]
    dts = [cases.stable_dt(c) for c in cs]
    b = solver.Batch(cs, autotune=False)
    assert b.info()["groups"] == 0
    for i, dt in enumerate(dts):
        b.set_dt(i, dt)
    b.step(9)
    got = [b.macros(i) for i in range(len(cs))]
    b.close()
    for i, c in enumerate(cs):
        s = solver.FvDVM(c, precision=solver.FP32_FP64MOM, pipeline=solver.PIPE_FUSED)
        s.set_dt(dts[i])
        s.evolution(9)
        want = s.macros()
        s.close()
        ref = Oracle(c)
        ref.step(dts[i], 9)
        oracle = ref.cell()
        for k in ("rho", "U", "T", "q"):
            assert np.array_equal(got[i][k], want[k]), (i, k)
            einf, el2 = rel_err(got[i][k], oracle[k])
            assert einf <= 1e-5 and el2 <= 1e-5, (i, k, einf, el2)
    with pytest.raises(solver.DugksError) as ei:
        solver.Batch(cs, persistent=True)
    assert ei.value.code == 3
