"""Known-answer test of the discrete-velocity generators against the
reference demo case's constant/Xis and constant/weights (tests/golden)."""
import json
import os

import numpy as np

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
