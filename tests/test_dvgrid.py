"""Known-answer test of the discrete-velocity generators against the
reference demo case's constant/Xis and constant/weights (tests/golden)."""
import json
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_gauss_hermite_matches_demo_case():
    from dugksfoam_gb300.dvgrid import gauss_hermite_half_range

    ref = json.load(open(os.path.join(HERE, "golden", "demo_cavity_dv.json")))
    x, w = gauss_hermite_half_range(ref["C"], ref["N"])
    X, W = np.array(ref["Xis"]), np.array(ref["weights"])
    assert np.abs(x - X).max() / np.abs(X).max() < 1e-13
    # the outermost weights carry exp(x^2) ~ 1e12: eigenvector round-off
    assert np.abs(w / W - 1).max() < 1e-9
    assert np.abs(w / W - 1)[2:-2].max() < 1e-12


def test_gauss_hermite_integrates_maxwellian_moments():
    from dugksfoam_gb300.dvgrid import gauss_hermite_half_range

    C = 337.196399395
    x, w = gauss_hermite_half_range(C, 28)
    f = np.exp(-(x / C) ** 2) / (np.sqrt(np.pi) * C)
    for k, exact in ((0, 1.0), (2, C * C / 2), (4, 3 * C ** 4 / 4)):
        assert abs((w * f * x ** k).sum() / exact - 1) < 1e-12


def test_command_line_writes_files_the_reader_takes(built_lib, tmp_path):
    """`python -m dugksfoam_gb300.dvgrid GH 337.196399395 28` (the reference's
    setDV.py interface) writes the demo case's grid; the case reader takes it."""
    from dugksfoam_gb300 import cases, dvgrid, foamio, solver

    case = cases.cavity2d(n=5, nxi=28)
    foamio.write_case(case, tmp_path)
    dvgrid.main(["GH", "337.196399395", "28", "--case", str(tmp_path)])
    ref = json.load(open(os.path.join(HERE, "golden", "demo_cavity_dv.json")))
    txt = (tmp_path / "constant" / "Xis").read_text()
    x = np.array([float(v) for v in txt[txt.index("(") + 1:txt.rindex(")")].split()])
    assert np.abs(x - np.array(ref["Xis"])).max() / np.abs(x).max() < 1e-13
    assert solver.inspect_case_dir(tmp_path)["n_xi_per_dim"] == 28


def test_command_line_refuses_nc_off_4z_plus_1(tmp_path):
    """setDV.py refuses NC grids with n != 4Z+1 (setDV.py:153-156); the other
    composite rules need --allow-other-rules."""
    from dugksfoam_gb300 import dvgrid

    with pytest.raises(SystemExit):
        dvgrid.main(["NC", "1348.0", "28", "--case", str(tmp_path)])
    xis, w = dvgrid.main(["NC", "1348.0", "29", "--case", str(tmp_path)])
    assert len(xis) == 29
    xis, w = dvgrid.main(["NC", "1348.0", "28", "--case", str(tmp_path), "--allow-other-rules"])
    assert len(xis) == 28 and abs(w.sum() - 2 * 1348.0) < 1e-9
