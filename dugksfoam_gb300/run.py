"""The dugksFoam application loop over the engine (src/dugksFoam.C:61-107).

    python -m dugksfoam_gb300.run <case_dir> [--precision fp32|fp64]

Reads the case directory (constant/polyMesh, constant/DVMProperties, Xis,
weights, 0/{rho,U,T}, system/controlDict) through dugks_create_from_case_dir,
then runs the reference's time loop:

  while runTime.run() and Uchange > convergeTol:
      CourantNo.H           dvm.getCoNum(CoNum, meanCoNum)
      setDeltaTvar.H        damped Courant-number time step (adjustTimeStep)
      runTime++             t += deltaT
      dvm.evolution()
      dvm.writeDFonCells()  at output times
      runTime.write()       at output times
      every convergeCheckSteps steps: the T, rho, U changes of dugksFoam.C:88-107

controlDict entries (readTimeControlsExplicit.H:39-52 and Time): startTime,
endTime, deltaT, writeControl (timeStep | runTime | adjustableRunTime),
writeInterval, timePrecision, adjustTimeStep, maxCo, maxDeltaT, convergeTol,
convergeCheckSteps.  One JSON line per convergence check goes to stdout.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import re
import sys

SMALL = 1.0e-15   # OpenFOAM SMALL
GREAT = 1.0e15    # OpenFOAM GREAT


def read_control_dict(case_dir):
    """Top-level ``key value;`` entries of system/controlDict as strings."""
    txt = open(os.path.join(case_dir, "system", "controlDict")).read()
    txt = re.sub(r"/\*.*?\*/", " ", txt, flags=re.S)
    txt = re.sub(r"//[^\n]*", " ", txt)
    txt = re.sub(r"FoamFile\s*\{[^}]*\}", " ", txt, flags=re.S)
    return {k: v.strip() for k, v in re.findall(r"^\s*([A-Za-z_]\w*)\s+([^;{}]+);", txt, flags=re.M)}


def _bool(v, default):
    if v is None:
        return default
    return v.strip().lower() in ("yes", "on", "true", "1")


def time_controls(cd):
    """The loop's controls with the reference's defaults (readTimeControlsExplicit.H)."""
    f = lambda k, d: float(cd[k]) if k in cd else d  # noqa: E731
    return dict(
        start=f("startTime", 0.0), end=f("endTime", GREAT), dt=f("deltaT", 0.0),
        write_control=cd.get("writeControl", "timeStep"), write_interval=f("writeInterval", 1.0),
        time_precision=int(f("timePrecision", 6)),
        adjust=_bool(cd.get("adjustTimeStep"), False), max_co=f("maxCo", 1.0), max_dt=f("maxDeltaT", GREAT),
        converge_tol=f("convergeTol", 1.0e-9), check_steps=max(1, int(f("convergeCheckSteps", 1))),
    )


def new_delta_t(dt, co, max_co, max_dt):
    """setDeltaTvar.H:34-50: reduction immediate, increase damped (at most 1.2x)."""
    fact = max_co / (co + SMALL)
    return min(min(min(fact, 1.0 + 0.1 * fact), 1.2) * dt, max_dt)


def adjust_to_write_time(dt, t, c, write_index):
    """Time::adjustDeltaT of OpenFOAM (called by Time::setDeltaT, which
    setDeltaTvar.H uses): under writeControl adjustableRunTime the step is
    stretched or shrunk so that a whole number of steps reaches the next
    write time, by at most 2x up and 5x down."""
    if c["write_control"] != "adjustableRunTime":
        return dt
    to_next = max(0.0, (write_index + 1) * c["write_interval"] - (t - c["start"]))
    n = to_next / dt - SMALL
    if n >= 2.0 ** 31 - 1:
        return dt
    new = to_next / (int(n) + 1)
    return min(new, 2.0 * dt) if new >= dt else max(new, 0.2 * dt)


def time_name(t, precision=6):
    """Time::timeName in the general format with timePrecision digits."""
    s = f"{t:.{precision}g}"
    return s


class OutputClock:
    """Time::outputTime for writeControl timeStep / runTime / adjustableRunTime."""

    def __init__(self, c):
        self.mode, self.interval, self.start = c["write_control"], c["write_interval"], c["start"]
        self.index = 0

    def __call__(self, step, t):
        if self.mode == "timeStep":
            return step % max(1, int(round(self.interval))) == 0
        k = int(math.floor((t - self.start) / self.interval + 1e-9))
        if k > self.index:
            self.index = k
            return True
        return False


def run(case_dir, precision, max_steps=None, out=None):
    from . import solver

    out = out if out is not None else sys.stdout
    cd = read_control_dict(case_dir)
    c = time_controls(cd)
    dvm = solver.FvDVM.from_case_dir(case_dir, precision=precision)
    dt = c["dt"] if c["dt"] > 0 else dvm.dt
    t, it, uchange = c["start"], 0, 1.0
    clock = OutputClock(c)
    # Time::run(): value() < endTime - 0.5 deltaT, with the step of the previous iteration
    while t < c["end"] - 0.5 * dt and uchange > c["converge_tol"]:
        co, mean_co = dvm.getCoNum()
        if c["adjust"]:
            dt = new_delta_t(dt, co, c["max_co"], c["max_dt"])
            dt = adjust_to_write_time(dt, t, c, clock.index)
        dvm.set_dt(dt)
        t += dt
        it += 1
        dvm.evolution(1)
        if clock(it, t):
            dvm.writeDFonCells(case_dir)
            dvm.write(case_dir, time_name(t, c["time_precision"]))
        if it % c["check_steps"] == 0:
            r = dvm.residual()
            uchange = r["U"]
            out.write(json.dumps(dict(step=it, time=t, deltaT=dt, CoNum=co, meanCoNum=mean_co, T_change=r["T"],
                                      rho_change=r["rho"], U_change=r["U"])) + "\n")
            out.flush()
        if max_steps is not None and it >= max_steps:
            break
    dvm.close()
    return it, t


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("case_dir")
    ap.add_argument("--precision", choices=["fp32", "fp64"], default="fp32")
    ap.add_argument("--max-steps", type=int, default=None, help="stop after this many steps")
    a = ap.parse_args(argv)
    from . import solver

    run(a.case_dir, solver.FP32_FP64MOM if a.precision == "fp32" else solver.FP64, a.max_steps)


if __name__ == "__main__":
    main()
