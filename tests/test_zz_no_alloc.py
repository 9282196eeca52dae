"""dugks_macros_noalloc: cell macros from caller-held device distributions,
without any device allocation inside the call.

Callers that cannot allocate (code inside a runtime that owns all device
memory, or a time loop that must not call cudaMalloc/cudaFree because they
synchronise the device) use this entry point.  It is checked through the C ABI
against the regular path -- dugks_get_macros after the engine's own moment
pass -- on two calls in a row: on FP64 and FP32 handles, 2D with h and 3D
without it, velocity sets whose size is not a multiple of the padded row
(n_dv != the padded row length), and with some outputs left NULL.  The device
buffers are allocated here by the test, never by the entry point: the device's
free memory is the same before and after the calls.  A case above the scratch
limit is refused before anything is launched.  This file is named so that
pytest collects it last.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu

MAX_CELLS = 262144  # the entry point's scratch limit (cells)
DUGKS_ERR_ARG = 1


def _device_buffers(s, g, h, with_h):
    import torch

    n = s.nCells
    gd = torch.from_numpy(np.ascontiguousarray(g)).cuda()
    hd = torch.from_numpy(np.ascontiguousarray(h)).cuda() if with_h else None
    out = {k: torch.full((n,) if k in ("rho", "T") else (n, 3), float("nan"), dtype=torch.float64, device="cuda")
           for k in ("rho", "U", "T", "q")}
    return gd, hd, out


def _ptr(t):
    return C.c_void_p(t.data_ptr()) if t is not None else C.c_void_p(None)


def _call(s, gd, hd, out, skip=()):
    import torch

    from dugksfoam_gb300 import solver

    lib = solver.load_library()
    torch.cuda.synchronize()
    rc = lib.dugks_macros_noalloc(s._h, _ptr(gd), _ptr(hd), *(C.c_void_p(None) if k in skip else _ptr(out[k])
                                                             for k in ("rho", "U", "T", "q")))
    s.synchronize()
    torch.cuda.synchronize()
    return rc, lib.dugks_last_error(s._h).decode()


CASES = {
    # name: (case factory, precision, tolerance)
    "fp64_2d": (lambda c: c.cavity2d(n=12, nxi=8), "FP64", 1e-12),
    "fp64_2d_nxi5": (lambda c: c.cavity2d(n=10, nxi=5), "FP64", 1e-12),
    "fp32_2d_nxi7": (lambda c: c.cavity2d(n=12, nxi=7), "FP32_FP64MOM", 1e-5),
    "fp64_3d_no_h": (lambda c: c.cavity3d(n=4, nxi=6), "FP64", 1e-12),
}


@pytest.mark.parametrize("name", list(CASES))
def test_macros_noalloc_matches_engine_macros(built_lib, name):
    import torch

    from dugksfoam_gb300 import cases, solver

    make, prec, tol = CASES[name]
    case = make(cases)
    s = solver.FvDVM(case, precision=getattr(solver, prec))
    info = s.info()
    with_h = bool(info["has_h"])
    assert info["n_dv_padded"] != info["n_dv"] or name in ("fp64_2d", "fp64_3d_no_h")
    s.set_dt(cases.stable_dt(case))
    s.evolution(2)
    g, h = s.dist()
    gd, hd, out = _device_buffers(s, g, h, with_h)
    assert _call(s, gd, hd, out)[0] == 0  # first call on the device: symbol address set-up
    for steps in (3, 2):  # two calls in a row, on two different states
        s.evolution(steps)
        want = s.macros()
        g, h = s.dist()
        gd.copy_(torch.from_numpy(g))
        if with_h:
            hd.copy_(torch.from_numpy(h))
        for t in out.values():
            t.fill_(float("nan"))
        free0 = torch.cuda.mem_get_info()[0]
        rc, msg = _call(s, gd, hd, out)
        assert rc == 0, msg
        assert torch.cuda.mem_get_info()[0] == free0  # the call allocated nothing
        for k in ("rho", "U", "T", "q"):
            einf, el2 = rel_err(out[k].cpu().numpy(), want[k])
            assert einf <= tol and el2 <= tol, (name, steps, k, einf, el2)
    # outputs left NULL are skipped; the others are still right
    for t in out.values():
        t.fill_(float("nan"))
    free0 = torch.cuda.mem_get_info()[0]
    rc, msg = _call(s, gd, hd, out, skip=("rho", "T"))
    assert rc == 0, msg
    assert torch.cuda.mem_get_info()[0] == free0
    assert torch.isnan(out["rho"]).all() and torch.isnan(out["T"]).all()
    for k in ("U", "q"):
        einf, el2 = rel_err(out[k].cpu().numpy(), want[k])
        assert einf <= tol and el2 <= tol, (name, "NULL rho/T", k, einf, el2)
    s.close()


def test_macros_noalloc_refuses_cases_above_its_limit(built_lib):
    """513^2 = 263169 cells > 262144: DUGKS_ERR_ARG before any launch (the
    outputs keep their contents)."""
    import torch

    from dugksfoam_gb300 import cases, solver

    case = cases.cavity2d(n=513, nxi=4)
    s = solver.FvDVM(case, precision=solver.FP64, pipeline=solver.PIPE_REFERENCE)
    assert s.nCells > MAX_CELLS
    n, nv = s.nCells, s.nDV
    gd = torch.zeros((n, nv), dtype=torch.float64, device="cuda")
    hd = torch.zeros((n, nv), dtype=torch.float64, device="cuda")
    out = {k: torch.full((n,) if k in ("rho", "T") else (n, 3), 7.0, dtype=torch.float64, device="cuda")
           for k in ("rho", "U", "T", "q")}
    rc, msg = _call(s, gd, hd, out)
    assert rc == DUGKS_ERR_ARG and "262144" in msg, (rc, msg)
    assert all(bool((t == 7.0).all()) for t in out.values())
    s.close()
