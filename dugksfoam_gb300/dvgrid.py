"""Discrete-velocity grid generators (the ``constant/Xis`` / ``constant/weights`` inputs).

Python 3 rewrite of dugksFoam's ``src/scripts/setDV.py`` (Python 2 only):

* ``gauss_hermite_half_range(C, N)`` -- the half-range Gauss--Hermite rule of
  ``setDV.py:83-114`` (``dvGH``).  The nodes/weights of the weight function
  exp(-x^2) on [0, inf) come from the three-term recurrence of the half-range
  Hermite polynomials and the Golub--Welsch eigenvalue method; the rule is
  mirrored to (-inf, inf), the weights are multiplied by exp(x^2) (so they
  integrate the plain distribution) and everything is scaled by C, the most
  probable molecular speed.  The recurrence is the published one the
  reference uses, so the demo case's ``Xis``/``weights`` files are a
  known-answer test for it.
* ``newton_cotes(xi_max, N)`` -- closed composite Newton--Cotes weights on N
  uniform nodes over [-xi_max, xi_max].  The reference ``dvNC``
  (``setDV.py:116-138``) only defines N = 4Z+1 (composite Boole rule,
  weights 7,32,12,32,14,...,7 x 4h/90) and refuses other N
  (``setDV.py:153-156``).  This generator reproduces ``dvNC`` exactly when
  (N-1) % 4 == 0 and otherwise uses the highest-order closed composite rule
  whose panel width divides N-1: Simpson 3/8 (3 | N-1), Simpson 1/3
  (2 | N-1), else the trapezoid rule.

Command line (the reference script's interface, ``setDV.py:140-160``), writing
``constant/Xis`` and ``constant/weights`` of the case in the current directory
(or ``--case``) as OpenFOAM lists in the same ``% 18.15e`` format:

    python -m dugksfoam_gb300.dvgrid GH 337.196399395 28
    python -m dugksfoam_gb300.dvgrid NC 1348.0 29
"""
from __future__ import annotations

import numpy as np

__all__ = ["gauss_hermite_half_range", "newton_cotes", "newton_cotes_rule", "write_dv_files", "main"]


def gauss_hermite_half_range(C: float, N: int):
    """Half-range Gauss--Hermite nodes and weights (setDV.py ``dvGH``).

    Returns (Xis, weights), each of length N (N even, >= 6).
    """
    if N % 2 != 0 or N < 6:
        raise ValueError("half-range Gauss-Hermite needs an even N >= 6")
    n = N // 2
    a = np.zeros(n)
    b = np.zeros(n)
    a[0] = 1.0 / np.sqrt(np.pi)
    a[1] = 2.0 / np.sqrt(np.pi) / (np.pi - 2.0)
    b[1] = a[0] / (a[0] + a[1]) / 2.0
    for i in range(2, n):
        b[i] = (i - 1) + 0.5 - b[i - 1] - a[i - 1] ** 2
        a[i] = (i ** 2 / 4.0 / b[i] - b[i - 1] - 0.5) / a[i - 1] - a[i - 1]
    off = np.sqrt(b[1:])
    jac = np.diag(a) + np.diag(off, 1) + np.diag(off, -1)
    nodes, vecs = np.linalg.eigh(jac)
    w = vecs[0, :] ** 2 * np.sqrt(np.pi) / 2.0
    order = np.argsort(nodes)
    nodes, w = nodes[order], w[order]
    xis = np.concatenate([-nodes[::-1], nodes])
    weights = np.concatenate([w[::-1], w])
    weights = weights * np.exp(xis ** 2) * C
    return xis * C, weights


def newton_cotes_rule(N: int) -> str:
    """Name of the closed composite rule used for N uniform nodes."""
    if N < 2:
        raise ValueError("need at least 2 nodes")
    p = N - 1
    if p % 4 == 0:
        return "boole"
    if p % 3 == 0:
        return "simpson38"
    if p % 2 == 0:
        return "simpson13"
    return "trapezoid"


_PANELS = {
    "boole": (4, np.array([7.0, 32.0, 12.0, 32.0, 7.0]) * 4.0 / 90.0),
    "simpson38": (3, np.array([1.0, 3.0, 3.0, 1.0]) * 3.0 / 8.0),
    "simpson13": (2, np.array([1.0, 4.0, 1.0]) / 3.0),
    "trapezoid": (1, np.array([0.5, 0.5])),
}


def newton_cotes(xi_max: float, N: int):
    """Uniform nodes on [-xi_max, xi_max] with closed composite N-C weights."""
    rule = newton_cotes_rule(N)
    xi_min = -xi_max
    dv = (xi_max - xi_min) / (N - 1)
    xis = np.array([xi_min + dv * i for i in range(N)])
    w = np.zeros(N)
    if rule == "boole":
        # same arithmetic as the reference dvNC, so N = 4Z+1 grids are bit-identical
        pattern = [14.0 / 90 * 4, 32.0 / 90 * 4, 12.0 / 90 * 4, 32.0 / 90 * 4]
        for i in range((N - 1) // 4):
            w[4 * i:4 * i + 4] = pattern
        w[0] = 7.0 / 90 * 4
        w[N - 1] = 7.0 / 90 * 4
        return xis, np.array([dv * wi for wi in w])
    width, panel = _PANELS[rule]
    for s in range(0, N - 1, width):
        w[s:s + width + 1] += panel
    return xis, w * dv


def _dv_file(obj, values):
    head = ("FoamFile\n{\n    version     2.0;\n    format      ascii;\n    class       dictionary;\n"
            f'    location    "constant";\n    object      {obj};\n}}\n\n')
    return head + f"{len(values)}\n(\n" + "".join("% 18.15e\n" % v for v in values) + ");"


def write_dv_files(case_dir, xis, weights):
    """constant/Xis and constant/weights of ``case_dir`` (the files fvDVM reads)."""
    import os

    d = os.path.join(case_dir, "constant")
    os.makedirs(d, exist_ok=True)
    with open(os.path.join(d, "Xis"), "w") as f:
        f.write(_dv_file("Xis", xis))
    with open(os.path.join(d, "weights"), "w") as f:
        f.write(_dv_file("weights", weights))


def main(argv=None):
    import argparse

    ap = argparse.ArgumentParser(description="Write constant/Xis and constant/weights (setDV.py).")
    ap.add_argument("rule", choices=["GH", "NC"], help="GH: half-range Gauss-Hermite; NC: Newton-Cotes")
    ap.add_argument("scale", type=float, help="GH: most probable speed C; NC: largest velocity xi_max")
    ap.add_argument("n", type=int, help="velocities per direction")
    ap.add_argument("--case", default=".", help="case directory (default: the current one)")
    ap.add_argument("--allow-other-rules", action="store_true",
                    help="NC with n != 4Z+1: composite Simpson-3/8, Simpson or trapezoid panels "
                         "(setDV.py refuses these n)")
    a = ap.parse_args(argv)
    if a.rule == "GH":
        if a.n % 2 != 0 or a.n < 7:  # the reference's check (setDV.py:145)
            ap.error("GH needs an even number of velocities, at least 8")
        xis, w = gauss_hermite_half_range(a.scale, a.n)
    else:
        if (a.n - 1) % 4 != 0 and not a.allow_other_rules:  # the reference's check (setDV.py:153-156)
            ap.error("NC needs 4Z+1 velocities per direction (--allow-other-rules for other n)")
        xis, w = newton_cotes(a.scale, a.n)
    write_dv_files(a.case, xis, w)
    return xis, w


if __name__ == "__main__":
    main()
