"""Gradient harness of the FP64 step (GPU): the hand-written adjoint against
the FP64 tangent-linear step (exact identity <grad, d> = dJ up to rounding),
both against central finite differences of the FP64 solver (h = 1e-3 K on the
lid temperatures, the objective's tolerance 1e-4), checkpoint invariance of
the adjoint, and the torch.autograd.Function binding.

Case: the adjoint configuration scaled down -- 8^2 quads with lid and bottom
wall patches, 8^2 DVs, lid temperatures 273 K + N(0, 5^2), 40 steps with the
objective averaged over the last 15, states checkpointed every 8 steps.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _setup(checkpoint_every=8):
    from dugksfoam_gb300 import cases, gradient

    base, Tw = gradient.adjoint_case(n=8, nxi=8)
    return gradient.Setup(case=base, dt=cases.stable_dt(base), n_steps=40, avg_first=25,
                          checkpoint_every=checkpoint_every), Tw


def test_adjoint_matches_tangent_linear(built_lib):
    from dugksfoam_gb300 import gradient

    setup, Tw = _setup()
    J, gTw, gs = gradient.adjoint(setup, Tw, 1.0)
    J0 = gradient.value(setup, Tw, 1.0)
    assert J == J0  # same FP64 forward
    rng = np.random.default_rng(1)
    for _ in range(2):
        dTw, ds = rng.standard_normal(len(Tw)), float(rng.standard_normal())
        Jt, dJ = gradient.tangent(setup, Tw, 1.0, dTw, ds)
        assert abs(Jt - J) <= 1e-12 * abs(J)
        dot = float(gTw @ dTw) + gs * ds
        assert abs(dot - dJ) <= 1e-9 * (abs(dJ) + np.abs(gTw).sum() + abs(gs)), (dot, dJ)


def test_tangent_and_adjoint_match_central_differences(built_lib):
    from dugksfoam_gb300 import gradient

    setup, Tw = _setup()
    J, gTw, gs = gradient.adjoint(setup, Tw, 1.0)
    h = 1e-3
    for k in (0, 3, 7):
        e = np.zeros(len(Tw))
        e[k] = 1.0
        fd = (gradient.value(setup, Tw + h * e, 1.0) - gradient.value(setup, Tw - h * e, 1.0)) / (2 * h)
        _, tl = gradient.tangent(setup, Tw, 1.0, e, 0.0)
        assert abs(fd) > 1e-3 * abs(J)  # a live sensitivity, not a zero
        assert abs(tl - fd) <= 1e-4 * abs(fd), (k, tl, fd)
        assert abs(gTw[k] - fd) <= 1e-4 * abs(fd), (k, gTw[k], fd)
    hs = 1e-5
    fd = (gradient.value(setup, Tw, 1.0 + hs) - gradient.value(setup, Tw, 1.0 - hs)) / (2 * hs)
    assert abs(fd) > 1e-3 * abs(J)
    assert abs(gs - fd) <= 1e-4 * abs(fd), (gs, fd)


def test_adjoint_independent_of_checkpoint_interval(built_lib, monkeypatch):
    """Same gradient for any checkpoint interval, with the per-step forward
    values kept for a segment or recomputed from the stored states."""
    from dugksfoam_gb300 import gradient

    ref = None
    for k, recompute in ((8, "0"), (12, "0"), (40, "0"), (8, "1"), (12, "1")):
        monkeypatch.setenv("DUGKS_ADJ_RECOMPUTE", recompute)
        setup, Tw = _setup(checkpoint_every=k)
        J, gTw, gs = gradient.adjoint(setup, Tw, 1.0)
        if ref is None:
            ref = (J, gTw, gs)
        else:
            assert J == ref[0] and np.array_equal(gTw, ref[1]) and gs == ref[2], (k, recompute)


def test_autograd_function(built_lib):
    torch = pytest.importorskip("torch")
    from dugksfoam_gb300 import gradient

    setup, Tw = _setup()
    t = torch.tensor(Tw, dtype=torch.float64, requires_grad=True)
    s = torch.tensor(1.0, dtype=torch.float64, requires_grad=True)
    J = gradient.WallObjective.apply(t, s, setup)
    (3.0 * J).backward()
    _, gTw, gs = gradient.adjoint(setup, Tw, 1.0)
    assert np.allclose(t.grad.numpy(), 3.0 * gTw, rtol=0, atol=0)
    assert float(s.grad) == 3.0 * gs
