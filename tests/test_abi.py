"""CPU checks of the C ABI: the library loads, exports every entry point the
header declares, and fails loudly (no CPU fallback) without a GPU."""
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    names = set()
    for fn in os.listdir(os.path.join(ROOT, "include", "dugks")):
        txt = open(os.path.join(ROOT, "include", "dugks", fn)).read()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        names |= set(re.findall(r"^\s*(?:int|const char\*|void)\s+(dugks_\w+)\s*\(", txt, flags=re.M))
    return names


def test_header_and_binding_agree():
    from dugksfoam_gb300 import solver

    assert _declared() == set(solver.EXPORTS)


def test_library_exports_every_declared_symbol(built_lib):
    import ctypes

    lib = ctypes.CDLL(built_lib)
    for name in _declared():
        assert hasattr(lib, name), name


def test_create_without_gpu_fails_loudly(built_lib):
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from dugksfoam_gb300 import cases, solver

    with pytest.raises(solver.DugksError) as ei:
        solver.FvDVM(cases.cavity2d(n=4, nxi=6))
    assert ei.value.code == 4


def test_invalid_case_is_rejected_before_device_use(built_lib):
    from dugksfoam_gb300 import cases, solver

    case = cases.cavity2d(n=4, nxi=6)
    case["mesh"] = dict(case["mesh"])
    own = case["mesh"]["owner"].copy()
    own[0] = 10**6
    case["mesh"]["owner"] = own
    with pytest.raises(solver.DugksError) as ei:
        solver.FvDVM(case)
    assert ei.value.code == 1
    assert "owner" in str(ei.value)


def test_dv_grid_rules():
    from dugksfoam_gb300.dvgrid import newton_cotes, newton_cotes_rule

    assert newton_cotes_rule(28) == "simpson38"
    assert newton_cotes_rule(32) == "trapezoid"
    assert newton_cotes_rule(41) == "boole"
    for n in (9, 13, 20, 28, 31, 32, 41):
        x, w = newton_cotes(1.0, n)
        assert abs(w.sum() - 2.0) < 1e-13
        assert abs((w * x * x).sum() - 2.0 / 3.0) < (0.05 if n < 12 else 0.01)
    x, w = newton_cotes(1600.0, 41)
    dv = 3200.0 / 40
    assert w[0] == dv * (7.0 / 90 * 4) and w[1] == dv * (32.0 / 90 * 4) and w[4] == dv * (14.0 / 90 * 4)
