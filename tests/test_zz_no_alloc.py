"""dugks_macros_noalloc: cell macros from caller-held device distributions,
without any device allocation inside the call.

Callers that cannot allocate (code inside a runtime that owns all device
memory, or a time loop that must not call cudaMalloc/cudaFree because they
synchronise the device) use this entry point.  It is checked through the C ABI
against the regular path -- dugks_get_macros after the engine's own moment
pass -- on two calls in a row, at the plain-FP64 tolerance.  The device
buffers are allocated here by the test, never by the entry point.  This file
is named so that pytest collects it last.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _call_noalloc(s, g, h):
    import torch

    from dugksfoam_gb300 import solver

    lib = solver.load_library()
    n = s.nCells
    gd = torch.from_numpy(np.ascontiguousarray(g)).cuda()
    hd = torch.from_numpy(np.ascontiguousarray(h)).cuda()
    out = {k: torch.full((n,) if k in ("rho", "T") else (n, 3), float("nan"), dtype=torch.float64, device="cuda")
           for k in ("rho", "U", "T", "q")}
    torch.cuda.synchronize()
    rc = lib.dugks_macros_noalloc(s._h, C.c_void_p(gd.data_ptr()), C.c_void_p(hd.data_ptr()),
                                  C.c_void_p(out["rho"].data_ptr()), C.c_void_p(out["U"].data_ptr()),
                                  C.c_void_p(out["T"].data_ptr()), C.c_void_p(out["q"].data_ptr()))
    assert rc == 0, lib.dugks_last_error(s._h).decode()
    s.synchronize()
    torch.cuda.synchronize()
    return {k: v.cpu().numpy() for k, v in out.items()}


def test_macros_noalloc_matches_engine_macros(built_lib):
    from dugksfoam_gb300 import cases, solver

    case = cases.cavity2d(n=12, nxi=8)
    s = solver.FvDVM(case, precision=solver.FP64, pipeline=solver.PIPE_REFERENCE)
    s.set_dt(cases.stable_dt(case))
    for steps in (3, 2):  # two calls in a row, on two different states
        s.evolution(steps)
        want = s.macros()
        g, h = s.dist()
        got = _call_noalloc(s, g, h)
        for k in ("rho", "U", "T", "q"):
            einf, el2 = rel_err(got[k], want[k])
            assert einf <= TOL and el2 <= TOL, (steps, k, einf, el2)
    s.close()
