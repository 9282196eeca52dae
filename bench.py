#!/usr/bin/env python3
"""Benchmark of the GB300 DUGKS engine (one JSON line on stdout).

Workload: the 2D unstructured lid-driven cavity -- ~100k seeded Delaunay
triangles (prisms), 32x32 discrete velocities, Kn 0.01 -- advanced with the
FP32-bulk / FP64-moment fused pipeline.  A "step" is one fvDVM::evolution()
(src/fvDVM/fvDVM/fvDVM.C:1086-1108) over every cell and velocity.

  value      cell*DV updates/s with the state resident in HBM (CUDA events on
             the engine's stream, max over ranks; the state, 819 MB of FP32 g
             and h, is larger than L2, so no flush is needed between steps)
  e2e        the same metric through the C ABI as dugksFoam's time loop uses
             the engine: per step dugks_get_conum (D2H), dugks_set_dt (H2D),
             dugks_step, dugks_get_macros into pinned host buffers (D2H)
  fp64_plain the plain FP64 pipeline on the same workload (the accuracy run)
  accuracy   field-normalised L-inf/L2 errors of rho, U, T, q of the FP32 step
             against the plain FP64 step after --accuracy-steps steps from the
             same initial state (gate 1e-5)
  roofline   the dominant kernel against measured HBM bandwidth: its
             algorithmic bytes (each array it reads or writes touched once)
             per launch over its CUDA-event launch time; step_frac is the
             whole step against the compulsory state traffic (read and write
             g~,h~ once: 16 B per cell*DV in FP32 with h, 8 B without)
  cpu_baseline the FP64 CPU oracle (a restatement of the reference step) on a
             bounded sample of the same workload, all host threads

--impl reference times that CPU restatement alone (the reference solver
itself needs OpenFOAM + MPI, which are not available).
Multi-GPU: the step does not shard across GPUs in this engine; --gpus N runs
N independent replicas (weak scaling), one per rank.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "cell*DV updates/s FP32+FP64-moment vs plain FP64, same GB300, <=1e-5 rel err"
UNIT = "cell*DV updates/s"


def alg_bytes(info):
    """Algorithmic bytes per launch of each FP32 kernel (each array read or
    written once): k_face_sides reads g~,h~ of every cell and writes the face
    values of every active face; k_cell_gather reads g~,h~ and the face values
    and writes g~new,h~new; k_face_macros moves O(faces) side data."""
    nd = 2 if info["has_h"] else 1
    V = info["n_dv"]
    nC, nA = info["n_cells"], info["n_internal_faces"] + info["n_wall_faces"]
    return {"k_face_sides": 4 * nd * V * (nC + nA), "k_cell_gather": 4 * nd * V * (2 * nC + nA),
            "k_face_macros": nA * (2 * 16 * 8 + 160)}


def rel_err(a, b):
    """Field-normalised L-inf and L2 errors (vector fields by the magnitude of the difference)."""
    import numpy as np

    a, b = np.asarray(a, float), np.asarray(b, float)
    if a.ndim == 2:
        d, r = np.linalg.norm(a - b, axis=1), np.linalg.norm(b, axis=1)
    else:
        d, r = np.abs(a - b), np.abs(b)
    return {"linf": float(d.max() / r.max()), "l2": float(np.linalg.norm(d) / np.linalg.norm(r))}


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons, sampled every 10 ms by one
    nvidia-smi process that runs across the timed region; mark() brackets the
    region and summary() keeps the samples inside it (or the nearest one on
    each side when the region is shorter than the sampling period)."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.samples = []  # (time, fields)
        self.t0 = self.t1 = None
        self._p = None
        self._t = None

    def _run(self):
        for line in self._p.stdout:
            f = [x.strip() for x in line.strip().split(",")]
            if len(f) == 7:
                self.samples.append((time.perf_counter(), f))

    def __enter__(self):
        try:
            self._p = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                        "--format=csv,noheader,nounits", "-lms", "10"],
                                       stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._run, daemon=True)
            self._t.start()
            deadline = time.perf_counter() + 5.0
            while not self.samples and time.perf_counter() < deadline:
                time.sleep(0.01)
        except Exception:
            self._p = None
        return self

    def mark(self, start):
        if start:
            self.t0 = time.perf_counter()
        else:
            self.t1 = time.perf_counter()
            time.sleep(0.05)  # let the sample after the region arrive

    def __exit__(self, *a):
        if self._p is not None:
            self._p.terminate()
            try:
                self._p.wait(timeout=5)
            except Exception:
                self._p.kill()
        if self._t is not None:
            self._t.join(timeout=5)

    def summary(self):
        smp = self.samples
        if self.t0 is not None and self.t1 is not None and smp:
            inside = [s for t, s in smp if self.t0 <= t <= self.t1]
            if not inside:
                before = [s for t, s in smp if t < self.t0][-1:]
                after = [s for t, s in smp if t > self.t1][:1]
                inside = before + after
            smp = inside
        else:
            smp = [s for _, s in smp]
        if not smp:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        num = lambda x: x.replace(".", "", 1).isdigit()
        sm = [float(s[0]) for s in smp if num(s[0])]
        mx = [float(s[1]) for s in smp if num(s[1])]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in smp for i in range(4) if s[3 + i].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(smp)}


def _dist():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def _allreduce_max(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist

    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def _barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def make_case(args):
    from dugksfoam_gb300 import cases

    if args.workload == "delaunay2d":
        case = cases.delaunay2d(n_interior=args.delaunay_interior, n_side=args.delaunay_side)
        return case, (f"delaunay2d: Delaunay triangles from {args.delaunay_interior} interior + "
                      f"4x{args.delaunay_side} boundary points (seed 0), 32x32 DV, Kn 0.01")
    if args.workload == "cavity2d":
        return cases.cavity2d(61, nxi=28), "cavity2d: 61x61 quads, 28x28 DV, Kn 0.075"
    if args.workload == "cavity3d":
        return cases.cavity3d(args.n3d, nxi=20), f"cavity3d: {args.n3d}^3 hexes, 20^3 DV, Kn 0.1"
    raise SystemExit(f"unknown workload {args.workload}")


def run_reference(args):
    """CPU restatement of the reference step (FP64 oracle) on a bounded sample."""
    world, rank, _ = _dist()
    if rank != 0:
        return
    from dugksfoam_gb300 import cases
    from oracle.oracle import Oracle

    case, desc = make_case(args)
    threads = os.cpu_count() or 1
    o = Oracle(case, threads=threads)
    dt = cases.case_dt(case)
    n = o.nC * o.nV
    for _ in range(args.warmup):
        o.step(dt, 1)
    t = time.perf_counter()
    for _ in range(args.steps):
        o.step(dt, 1)
    el = time.perf_counter() - t
    v = n * args.steps / el
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": el / args.steps * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": desc, "cells": o.nC, "dvs": o.nV},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"{args.steps} full steps of the workload (FP64 oracle, OpenMP)"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def cpu_baseline(case, seconds=15.0):
    from dugksfoam_gb300 import cases
    from oracle.oracle import Oracle

    threads = os.cpu_count() or 1
    o = Oracle(case, threads=threads)
    dt = cases.case_dt(case)
    o.step(dt, 1)
    steps, t0 = 0, time.perf_counter()
    while True:
        o.step(dt, 1)
        steps += 1
        if time.perf_counter() - t0 > seconds or steps >= 20:
            break
    el = time.perf_counter() - t0
    return {"value": o.nC * o.nV * steps / el, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{steps} full steps of the same workload after 1 warm-up step (FP64 oracle, OpenMP)"}


def run_engine(args):
    import torch

    from dugksfoam_gb300 import cases, solver

    world, rank, local = _dist()
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", init_method="env://")
    torch.cuda.set_device(local)
    case, desc = make_case(args)
    dt = cases.case_dt(case)
    s = solver.FvDVM(case, precision=solver.FP32_FP64MOM, pipeline=solver.PIPE_FUSED, device=local)
    stream = torch.cuda.Stream()
    s.set_stream(stream.cuda_stream)
    s.set_dt(dt)
    info = s.info()
    n_upd = s.nCells * s.nDV
    # warm-up
    s.evolution(args.warmup)
    s.synchronize()
    # ---- device-resident throughput (CUDA events on the engine's stream)
    _barrier(world)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk, torch.cuda.stream(stream):
        clk.mark(True)
        e0.record(stream)
        s.evolution(args.steps)
        e1.record(stream)
        e1.synchronize()
        clk.mark(False)
    torch.cuda.synchronize()
    _barrier(world)
    ms = e0.elapsed_time(e1)
    ms = _allreduce_max(ms, world)
    s.synchronize()
    value = n_upd * args.steps * world / (ms / 1e3)
    # ---- per-kernel times (CUDA events around each launch) for the roofline
    prof = s.profile(3)
    # ---- end to end through the C ABI with host buffers (pinned)
    nC = s.nCells
    hb = {k: torch.empty(sz, dtype=torch.float64, pin_memory=True).numpy()
          for k, sz in (("rho", nC), ("U", 3 * nC), ("T", nC), ("q", 3 * nC))}
    ek = max(3, args.steps // 2)
    _barrier(world)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(ek):
        s.getCoNum()
        s.set_dt(dt)
        s.evolution(1)
        s.macros_into(hb["rho"], hb["U"], hb["T"], hb["q"])
    t_e2e = _allreduce_max(time.perf_counter() - t0, world)
    e2e = n_upd * ek * world / t_e2e
    d2h = sum(a.nbytes for a in hb.values()) + 16
    # ---- plain FP64 pipeline on the same workload (rank 0 only), then the
    # accuracy of the FP32 step against it: a fresh FP32 handle and the FP64
    # handle advance the same number of steps from the same initial state
    fp64 = None
    accuracy = None
    if rank == 0 and not args.skip_fp64:
        s64 = solver.FvDVM(case, precision=solver.FP64, pipeline=solver.PIPE_REFERENCE, device=local)
        st64 = torch.cuda.Stream()
        s64.set_stream(st64.cuda_stream)
        s64.set_dt(dt)
        s64.evolution(1)
        s64.synchronize()
        n_acc = max(args.accuracy_steps, 0)
        k64 = max(2, args.steps // 5, n_acc - 1)
        a0, a1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a0.record(st64)
        s64.evolution(k64)
        a1.record(st64)
        a1.synchronize()
        ms64 = a0.elapsed_time(a1)
        fp64 = {"value": n_upd * k64 / (ms64 / 1e3), "ms_per_step": ms64 / k64, "steps": k64,
                "pipeline": "reference (one FP64 kernel per fvDVM pass)"}
        if n_acc > 0:
            m64 = s64.macros()
            s32 = solver.FvDVM(case, precision=solver.FP32_FP64MOM, pipeline=solver.PIPE_FUSED, device=local)
            s32.set_dt(dt)
            s32.evolution(k64 + 1)
            m32 = s32.macros()
            s32.close()
            accuracy = {"steps": k64 + 1, "against": "plain FP64 pipeline, same initial state",
                        "norm": "field-normalised; vectors by the magnitude of the difference", "gate": 1e-5}
            for k in ("rho", "U", "T", "q"):
                accuracy[k] = rel_err(m32[k], m64[k])
            accuracy["max"] = max(max(accuracy[k].values()) for k in ("rho", "U", "T", "q"))
            accuracy["pass"] = accuracy["max"] <= accuracy["gate"]
        s64.close()
    if rank != 0:
        return
    peak, peak_kind = _peaks()
    dom = max(prof, key=prof.get)
    alg = alg_bytes(info)
    achieved = alg[dom] / (prof[dom] / 1e3) / 1e9
    step_bytes = 4 * (2 if info["has_h"] else 1) * 2  # read + write g~(,h~) once, FP32
    traffic = None
    tfile = os.path.join(ROOT, "profiles", "traffic_per_cell_dv.json")
    if os.path.exists(tfile):  # ncu DRAM bytes per cell*DV of each kernel (small-case capture)
        try:
            tb = json.load(open(tfile)).get(args.workload, {}).get(dom)
            traffic = tb * n_upd if tb else None
        except Exception:
            traffic = None
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 distributions, f64 moments", "data": "synthetic",
        "config": {"workload": desc, "cells": s.nCells, "dvs": s.nDV, "dv_padded": info["n_dv_padded"],
                   "state_bytes": int((2 if info["has_h"] else 1) * 4 * s.nCells * info["n_dv_padded"]),
                   "l2": "state larger than the 129 MB L2; no flush needed", "dt": dt,
                   "parallelism": f"replicas x{world}"},
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_kind": peak_kind, "traffic": traffic,
                     "alg_bytes": alg[dom],
                     "step_bytes_per_cell_dv": step_bytes,
                     "step_frac": step_bytes * value / world / 1e9 / peak},
        "kernels_ms": prof,
        "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": 8, "d2h_bytes_per_step": d2h},
        "gpu_launches": s.launches_per_step() * args.steps,
        "clocks": clk.summary(),
        "fp64_plain": fp64,
        "speedup_vs_fp64_plain": (value / world / fp64["value"]) if fp64 else None,
        "accuracy": accuracy,
    }
    s.close()
    if not args.skip_cpu:
        line["cpu_baseline"] = cpu_baseline(case, seconds=args.cpu_seconds)
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="engine", choices=["engine", "reference"])
    ap.add_argument("--workload", default="delaunay2d", choices=["delaunay2d", "cavity2d", "cavity3d"])
    ap.add_argument("--delaunay-interior", type=int, default=49200,
                    help="interior points of the delaunay2d mesh (49200 -> ~100k triangles)")
    ap.add_argument("--delaunay-side", type=int, default=400, help="points per side of the delaunay2d boundary")
    ap.add_argument("--n3d", type=int, default=48, help="hexes per side of the cavity3d mesh")
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--skip-fp64", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--accuracy-steps", type=int, default=500,
                    help="steps of the FP32-vs-FP64 accuracy check after the timed run (0: none)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_engine(args)


if __name__ == "__main__":
    main()
