"""TEST INFRASTRUCTURE ONLY: run the FP64 CPU oracle (the restatement of the
reference step) on a named workload for many steps, logging the range of the
macroscopic fields every --log steps (one JSON line each) and saving the cell
fields every --every steps, until the step count or a non-finite /
non-positive state.  Used to check long runs of the GPU engine against the
oracle and to confirm where the reference scheme itself diverges.

    python oracle/run_case.py --workload delaunay2d --steps 2000 --every 250 --out <dir>
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))


def main(argv=None):
    from dugksfoam_gb300 import cases
    from oracle.oracle import Oracle

    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--workload", default="delaunay2d", choices=["delaunay2d", "cavity2d"])
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--every", type=int, default=250, help="save the cell fields every this many steps")
    ap.add_argument("--log", type=int, default=50)
    ap.add_argument("--threads", type=int, default=os.cpu_count() or 1)
    ap.add_argument("--out", required=True)
    a = ap.parse_args(argv)
    case = cases.delaunay2d() if a.workload == "delaunay2d" else cases.cavity2d(61, nxi=28)
    dt = cases.case_dt(case)
    o = Oracle(case, threads=a.threads)
    os.makedirs(a.out, exist_ok=True)
    print(json.dumps(dict(workload=a.workload, cells=o.nC, dvs=o.nV, dt=dt, threads=a.threads)), flush=True)
    t0 = time.time()
    for s in range(1, a.steps + 1):
        o.step(dt, 1)
        if s % a.log and s % a.every:
            continue
        c = o.cell()
        qn = np.linalg.norm(c["q"], axis=1)
        ok = bool(np.isfinite(c["q"]).all() and np.isfinite(c["T"]).all() and c["rho"].min() > 0 and c["T"].min() > 0)
        print(json.dumps(dict(step=s, seconds=round(time.time() - t0, 1), rho_min=float(c["rho"].min()),
                              T_min=float(c["T"].min()), T_max=float(c["T"].max()),
                              U_max=float(np.linalg.norm(c["U"], axis=1).max()), q_max=float(qn.max()),
                              q_argmax=int(qn.argmax()), finite=ok)), flush=True)
        if s % a.every == 0:
            np.savez(os.path.join(a.out, f"{a.workload}_{s}.npz"), **c)
        if not ok:
            break


if __name__ == "__main__":
    main()
