"""Generates the golden fixtures in tests/golden/ (run from the repo root).

* ``cavity61_2000.npz`` -- FP64 oracle fields (rho, U, T, q, tau) after the
  stated 2000 steps of the 61x61-quad, 28x28-DV lid-driven cavity
  (Kn 0.075, dt = 0.5 dx / (sqrt(2) xi_max)).  This is the CPU-runnable case's
  full run; GPU parity at the stated step count is checked against it.
* ``demo_cavity_dv.json`` -- the reference demo case's constant/Xis and
  constant/weights (demo/cavity/constant/, produced by the reference's
  ``setDV.py GH 337.196399395 28``, doc/demo.tex:25-30): the known-answer
  test of the half-range Gauss-Hermite generator.  Read from the reference
  checkout when it is present.

Usage: python tests/golden/make_golden.py [--cavity] [--dv]
"""
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)


def cavity():
    from dugksfoam_gb300 import cases
    from oracle.oracle import Oracle

    case = cases.cavity2d(n=61, nxi=28)
    dt = cases.stable_dt(case)
    o = Oracle(case)
    t = time.time()
    o.step(dt, 2000)
    c = o.cell()
    np.savez_compressed(os.path.join(HERE, "cavity61_2000.npz"), dt=dt, steps=2000, **c)
    print(f"cavity61_2000: {time.time() - t:.1f}s  T range {c['T'].min():.4f}..{c['T'].max():.4f}")


def _read_list(path):
    txt = open(path).read()
    body = txt[txt.index("FoamFile"):]
    body = body[body.index("}") + 1:]
    n = int(body.split("(")[0].split()[-1])
    vals = [float(v) for v in body.split("(")[1].split(")")[0].split()]
    assert len(vals) == n
    return vals


def dv(ref_root=None):
    """The demo case's Xis/weights from the reference checkout (DUGKS_REFERENCE_ROOT)."""
    ref_root = ref_root or os.environ["DUGKS_REFERENCE_ROOT"]
    d = os.path.join(ref_root, "demo", "cavity", "constant")
    out = dict(C=337.196399395, N=28, Xis=_read_list(os.path.join(d, "Xis")),
               weights=_read_list(os.path.join(d, "weights")),
               source="demo/cavity/constant/{Xis,weights} of zhulianhua/dugksFoam")
    json.dump(out, open(os.path.join(HERE, "demo_cavity_dv.json"), "w"), indent=1)
    print("demo_cavity_dv.json written")


if __name__ == "__main__":
    args = sys.argv[1:] or ["--dv", "--cavity"]
    if "--dv" in args:
        dv()
    if "--cavity" in args:
        cavity()
