"""Accuracy of the FP32 / FP64-moment step against the plain FP64 step on a
workload, after a stated number of steps: field-normalised L-inf and L2
errors of rho, U, T, q (vector fields by the magnitude of the difference).
The FP64 reference is the plain FP64 GPU pipeline, which the parity tests pin
to the CPU oracle at 1e-12.  One JSON line on stdout."""
from __future__ import annotations

import argparse
import json
import time

import numpy as np


def rel_err(a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    if a.ndim == 2:
        d, r = np.linalg.norm(a - b, axis=1), np.linalg.norm(b, axis=1)
    else:
        d, r = np.abs(a - b), np.abs(b)
    return dict(linf=float(d.max() / r.max()), l2=float(np.linalg.norm(d) / np.linalg.norm(r)))


def main(argv=None):
    from . import cases, solver

    ap = argparse.ArgumentParser(description=__doc__)
    ap.add_argument("--workload", default="delaunay2d",
                    choices=["delaunay2d", "cavity2d", "cavity3d", "cavity128", "batch"])
    ap.add_argument("--instances", default="0-7", help="batch: instance range a-b of the seeded cavities")
    ap.add_argument("--steps", type=int, default=5000)
    ap.add_argument("--n3d", type=int, default=48)
    ap.add_argument("--at", default="", help="comma-separated step counts at which to report as well (trajectory)")
    ap.add_argument("--delaunay-interior", type=int, default=49200)
    ap.add_argument("--delaunay-side", type=int, default=400)
    ap.add_argument("--save", default="", help="directory: write both runs' cell fields at every mark (npz)")
    a = ap.parse_args(argv)
    if a.workload == "batch":
        return run_batch(a)
    case = {"delaunay2d": lambda: cases.delaunay2d(n_interior=a.delaunay_interior, n_side=a.delaunay_side),
            "cavity2d": lambda: cases.cavity2d(61, nxi=28),
            "cavity128": lambda: cases.cavity2d(128, Kn=0.075, nxi=32, bottom_patch=True),
            "cavity3d": lambda: cases.cavity3d(a.n3d, nxi=20)}[a.workload]()
    dt = cases.case_dt(case)
    marks = sorted({int(x) for x in a.at.split(",") if x} | {a.steps})
    runs = {}
    for name, prec, pipe in (("fp32", solver.FP32_FP64MOM, solver.PIPE_FUSED), ("fp64", solver.FP64, solver.PIPE_REFERENCE)):
        s = solver.FvDVM(case, precision=prec, pipeline=pipe)
        s.set_dt(dt)
        runs[name] = s
    done = 0
    for n in marks:
        out = dict(workload=a.workload, steps=n, dt=dt, cells=runs["fp32"].nCells, dvs=runs["fp32"].nDV)
        fields = {}
        for name, s in runs.items():
            t = time.perf_counter()
            try:
                s.evolution(n - done)
                fields[name] = s.macros()
            except solver.DugksError as e:  # a run that blew up: NaN/Inf or non-positive rho/T
                out[f"failed_{name}"] = str(e)
            out[f"seconds_{name}"] = time.perf_counter() - t
        done = n
        if len(fields) == 2:
            out["error_fp32_vs_fp64"] = {k: rel_err(fields["fp32"][k], fields["fp64"][k]) for k in ("rho", "U", "T", "q")}
        if a.save and fields:
            import os

            import numpy as np

            os.makedirs(a.save, exist_ok=True)
            np.savez(os.path.join(a.save, f"{a.workload}_{n}.npz"),
                     **{f"{k}_{name}": f[k] for name, f in fields.items() for k in ("rho", "U", "T", "q")})
        print(json.dumps(out), flush=True)
        if len(fields) < 2:
            break
    for s in runs.values():
        s.close()


def run_batch(a):
    """The batched cavities (the seeded instances of the batched runner),
    advanced together by the batched FP32 engine, each against the same case
    run alone on the plain FP64 pipeline; one JSON line per instance."""
    from . import cases, solver

    lo, hi = (int(x) for x in a.instances.split("-"))
    inst = cases.batch_instances(hi + 1, a.steps)[lo:hi + 1]
    cs = [cases.batch_case(i) for i in inst]
    dts = [cases.stable_dt(c) for c in cs]
    b = solver.Batch(cs, autotune=False)
    for i, dt in enumerate(dts):
        b.set_dt(i, dt)
    b.step(a.steps)
    got = [b.macros(i) for i in range(len(cs))]
    b.close()
    for i, c in enumerate(cs):
        s = solver.FvDVM(c, precision=solver.FP64, pipeline=solver.PIPE_REFERENCE)
        s.set_dt(dts[i])
        s.evolution(a.steps)
        want = s.macros()
        out = dict(workload="batch", instance=lo + i, N=inst[i]["N"], M=inst[i]["M"], Kn=inst[i]["Kn"],
                   steps=a.steps, cells=s.nCells, dvs=s.nDV,
                   error_fp32_vs_fp64={k: rel_err(got[i][k], want[k]) for k in ("rho", "U", "T", "q")})
        s.close()
        print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
