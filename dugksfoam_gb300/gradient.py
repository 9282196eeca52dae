"""Gradient harness: wall-flux objective of the DUGKS step as a
``torch.autograd.Function`` over the engine's C-ABI adjoint.

The objective (config of the 128^2 adjoint case): the mean over the last
steps of the lid heat flux through the lid, sum_w S_w . qWall_w, plus the
bottom-wall shear, sum_w |S_w| stressWall_w,xy.  Parameters: the wall
temperature of each lid face and the relaxation-time scale s (mu_ref -> s mu_ref).

``WallObjective.apply(Tw_lid, s, setup)`` returns J (a 0-d tensor); its
backward multiplies the incoming gradient by dJ/dTw_lid and dJ/ds, which the
forward computes with dugks_objective_adjoint (FP64 step, checkpointed every
``setup.checkpoint_every`` steps).  Torch is used for the tensor plumbing only;
no torch operation enters the derivative.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from . import cases, solver


@dataclass
class Setup:
    case: dict            # base case (cases.make_case dict), lid / bottom patches present
    dt: float
    n_steps: int
    avg_first: int
    q_patch: str = "movingWall"
    stress_patch: str = "bottomWall"
    checkpoint_every: int = 100


def patch_index(case, name):
    for i, p in enumerate(case["mesh"]["patches"]):
        if p["name"] == name:
            return i
    raise KeyError(name)


def wall_slice(case, name):
    """Wall-face range (wall order = patch order) and boundary-face range of a patch."""
    m = case["mesh"]
    nI = len(m["neighbour"])
    w0 = 0
    for p in m["patches"]:
        if p["name"] == name:
            return slice(w0, w0 + p["nFaces"]), slice(p["startFace"] - nI, p["startFace"] - nI + p["nFaces"])
        if p["type"] == "wall":
            w0 += p["nFaces"]
    raise KeyError(name)


def parametrised_case(setup: Setup, Tw_lid, s):
    """Copy of the base case with the lid wall temperatures and mu_ref scaled by s."""
    c = dict(setup.case)
    c["Tb"] = np.array(setup.case["Tb"], dtype=np.float64, copy=True)
    _, bsl = wall_slice(setup.case, setup.q_patch)
    c["Tb"][bsl] = np.asarray(Tw_lid, np.float64)
    c["gas"] = dict(setup.case["gas"])
    c["gas"]["muRef"] = setup.case["gas"]["muRef"] * float(s)
    return c


def objective_handle(setup: Setup, Tw_lid, s, precision=solver.FP64):
    h = solver.FvDVM(parametrised_case(setup, Tw_lid, s), precision=precision)
    h.set_dt(setup.dt)
    return h


def _desc(setup):
    return dict(n_steps=setup.n_steps, avg_first=setup.avg_first,
                q_patch=patch_index(setup.case, setup.q_patch) if setup.q_patch else -1,
                stress_patch=patch_index(setup.case, setup.stress_patch) if setup.stress_patch else -1,
                checkpoint_every=setup.checkpoint_every)


def value(setup: Setup, Tw_lid, s):
    h = objective_handle(setup, Tw_lid, s)
    try:
        return h.objective_value(**_desc(setup))
    finally:
        h.close()


def adjoint(setup: Setup, Tw_lid, s):
    """(J, dJ/dTw_lid, dJ/ds) by the adjoint."""
    h = objective_handle(setup, Tw_lid, s)
    try:
        J, gTw, gmu = h.objective_adjoint(**_desc(setup))
    finally:
        h.close()
    wsl, _ = wall_slice(setup.case, setup.q_patch)
    return J, gTw[wsl], gmu / float(s)  # handle derivative is per unit of its own mu scale


def tangent(setup: Setup, Tw_lid, s, dTw_lid, ds):
    """(J, dJ) along (dTw_lid, ds) by the FP64 tangent-linear step."""
    h = objective_handle(setup, Tw_lid, s)
    try:
        nW = h.info()["n_wall_faces"]
        d = np.zeros(nW)
        wsl, _ = wall_slice(setup.case, setup.q_patch)
        d[wsl] = dTw_lid
        return h.objective_tangent(d, ds / float(s), **_desc(setup))
    finally:
        h.close()


try:
    import torch

    class WallObjective(torch.autograd.Function):
        """J(Tw_lid, s) with the adjoint gradient (C ABI) as its backward."""

        @staticmethod
        def forward(ctx, Tw_lid, s, setup):
            J, gTw, gs = adjoint(setup, Tw_lid.detach().cpu().double().numpy(), float(s))
            ctx.save_for_backward(torch.as_tensor(gTw, dtype=Tw_lid.dtype), torch.as_tensor(gs, dtype=Tw_lid.dtype))
            return torch.as_tensor(J, dtype=Tw_lid.dtype)

        @staticmethod
        def backward(ctx, gJ):
            gTw, gs = ctx.saved_tensors
            return gJ * gTw, gJ * gs, None

except ImportError:  # torch is optional for the plain-numpy entry points
    WallObjective = None


def adjoint_case(n=128, nxi=32, Kn=0.075, seed=0, sigma=5.0):
    """The 128^2 adjoint case: lid and bottom wall patches, lid temperatures
    273 K + N(0, sigma^2) from default_rng(seed)."""
    base = cases.cavity2d(n=n, Kn=Kn, nxi=nxi, bottom_patch=True)
    nlid = wall_slice(base, "movingWall")[0].stop - wall_slice(base, "movingWall")[0].start
    Tw = 273.0 + sigma * np.random.default_rng(seed).standard_normal(nlid)
    return base, Tw


def main(argv=None):
    """Adjoint case run: J, the adjoint gradient, its agreement with the
    tangent-linear step and (optionally) central differences, and the cost of
    the adjoint against one FP64 forward.  One JSON line on stdout."""
    import argparse
    import json
    import time

    ap = argparse.ArgumentParser(description=main.__doc__)
    ap.add_argument("--n", type=int, default=128)
    ap.add_argument("--nxi", type=int, default=32)
    ap.add_argument("--steps", type=int, default=3000)
    ap.add_argument("--window", type=int, default=500)
    ap.add_argument("--checkpoint-every", type=int, default=100)
    ap.add_argument("--fd", type=int, default=0, help="number of lid faces checked by central differences")
    a = ap.parse_args(argv)
    base, Tw = adjoint_case(n=a.n, nxi=a.nxi)
    setup = Setup(case=base, dt=cases.stable_dt(base), n_steps=a.steps, avg_first=a.steps - a.window,
                  checkpoint_every=a.checkpoint_every)
    t0 = time.perf_counter()
    J0 = value(setup, Tw, 1.0)
    t1 = time.perf_counter()
    J, gTw, gs = adjoint(setup, Tw, 1.0)
    t2 = time.perf_counter()
    d = np.random.default_rng(1).standard_normal(len(Tw))
    Jt, dJ = tangent(setup, Tw, 1.0, d, 1.0)
    t3 = time.perf_counter()
    out = dict(case=f"{a.n}^2 quads, {a.nxi}^2 DVs, {a.steps} steps, objective over the last {a.window}, "
                    f"checkpoint every {a.checkpoint_every}",
               J=J, J_forward=J0, dJ_ds=gs, dJ_dTw_norm=float(np.linalg.norm(gTw)),
               adjoint_vs_tangent=abs(float(gTw @ d) + gs - dJ) / abs(dJ),
               seconds=dict(forward=t1 - t0, adjoint=t2 - t1, tangent=t3 - t2),
               adjoint_over_forward=(t2 - t1) / (t1 - t0))
    if a.fd:
        h, errs = 1e-3, []
        for k in np.linspace(0, len(Tw) - 1, a.fd).astype(int):
            e = np.zeros(len(Tw))
            e[k] = 1.0
            fd = (value(setup, Tw + h * e, 1.0) - value(setup, Tw - h * e, 1.0)) / (2 * h)
            errs.append(abs(gTw[k] - fd) / abs(fd))
        out["fd_rel_err_max"] = max(errs)
    print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
