"""Batched-cases run: the 64 seeded 2D cavities (uneven N x N meshes with
N in 32..128, M x M velocity grids with M in 16..40, Kn log-uniform in
[0.01, 1], lid 10..100 m/s, Tw 250..350 K), FP32 bulk / FP64 moments,
advanced together with the batched engine (one launch per pass over all
cases, two steps per CUDA graph, autotuned DVs per lane and tile cap), and the
same cases stepped one after another as separate engines, and the persistent
kernel (every pass and step of every case in one cooperative launch), for
comparison.
One JSON line on stdout."""
from __future__ import annotations

import argparse
import json
import time


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__)
    ap.add_argument("--cases", type=int, default=64)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--separate-steps", type=int, default=100, help="steps of the one-engine-per-case comparison")
    ap.add_argument("--no-autotune", action="store_true")
    a = ap.parse_args(argv)

    import torch

    from . import cases, solver

    inst = cases.batch_instances(a.cases, a.steps)
    cs = [cases.batch_case(i) for i in inst]
    dts = [cases.stable_dt(c) for c in cs]
    t0 = time.perf_counter()
    b = solver.Batch(cs, autotune=not a.no_autotune)
    t_build = time.perf_counter() - t0
    for i, dt in enumerate(dts):
        b.set_dt(i, dt)
    info = b.info()
    b.step(4)
    b.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    e0.record()
    b.step(a.steps)
    b.synchronize()
    e1.record()
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    ms = wall * 1e3  # the batch runs on its own stream: wall time around a synchronised region
    ok = all(float(b.macros(i)["rho"].min()) > 0 for i in range(len(cs)))
    b.close()
    # the persistent kernel: every pass and step in one cooperative launch
    p = solver.Batch(cs, persistent=True)
    for i, dt in enumerate(dts):
        p.set_dt(i, dt)
    p.step(4)
    p.synchronize()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    p.step(a.steps)
    p.synchronize()
    wall_p = time.perf_counter() - t0
    ok_p = all(float(p.macros(i)["rho"].min()) > 0 for i in range(len(cs)))
    p.close()
    # separate engines, one case after another per step
    eng = []
    for i, c in enumerate(cs):
        s = solver.FvDVM(c, precision=solver.FP32_FP64MOM, pipeline=solver.PIPE_FUSED)
        s.set_dt(dts[i])
        eng.append(s)
    for s in eng:
        s.evolution(2)
    for s in eng:
        s.synchronize()
    t0 = time.perf_counter()
    for _ in range(a.separate_steps):
        for s in eng:
            s.evolution(1)
    for s in eng:
        s.synchronize()
    sep = (time.perf_counter() - t0) / a.separate_steps
    for s in eng:
        s.close()
    cdv = info["cell_dv"]
    print(json.dumps(dict(
        workload=f"{a.cases} seeded 2D cavities (N 32..128, M 16..40), FP32 / FP64-moment",
        cells=info["cells"], cell_dv_per_step=cdv, steps=a.steps,
        batched=dict(ms_per_step=ms / a.steps, cell_dv_per_s=cdv * a.steps / (ms / 1e3),
                     dv_per_lane=info["dv_per_lane"], tile_cap=info["tile_cap"], tuned=info["tuned"],
                     launches_per_step=info["launches_per_step"], steps_per_graph=info["steps_per_graph"],
                     build_and_tune_s=t_build, finite=ok),
        persistent=dict(ms_per_step=wall_p * 1e3 / a.steps, cell_dv_per_s=cdv * a.steps / wall_p,
                        launches=1, finite=ok_p),
        separate_engines=dict(ms_per_step=sep * 1e3, cell_dv_per_s=cdv / sep, launches_per_step=3 * a.cases),
        speedup=(sep * 1e3) / (ms / a.steps))), flush=True)


if __name__ == "__main__":
    main()
