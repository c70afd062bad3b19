"""Throughput of the single-world configurations on the GPU, beside the CPU restatement of the
reference step on one host core, on the same seeded scenes.

  python configs_report.py [--configs 1,2,5] [--cpu-seconds 15] [--threads 128,256,512]

Configurations (the batched one is bench.py's):
  1  the 210-box pyramid on an edge ground, sleep on (the reference default), 600 steps;
  2  10,000 circles and convex polygons dropped into a 200 m edge box, sleep off, steps 1..200;
  5  65,536 bodies with 512 revolute chains of 16 links in a 300 m container spinning at 0.05 rad/s,
     sleep off, steps 1..60.

GPU: one world per handle, the plain (reference-order, bit-exact) and the graph-coloured solver,
8/3 iterations, one CTA of each --threads width (every width computes the same bits), every step
replayed from the captured graph and timed in blocks of 50 steps with CUDA events on the handle's
stream; body-steps/s over the timed steps. CPU: the oracle's restatement of b2World::Step (plain order) with glibc's sinf/cosf (the
reference's own trig) on one thread, stepped from the same initial state for as many of the same
steps as fit in --cpu-seconds. Prints one JSON line per configuration. A CPU-baseline reporter like
bench.py's CPU leg: it sits beside bench.py, outside the package, because it runs the oracle.
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))

DT, VI, PI = 1.0 / 60.0, 8, 3


def scene(cfg: int):
    from box2dpp_gb300 import scenes

    if cfg == 1:
        return scenes.config1(), 600
    if cfg == 2:
        return scenes.config2(10000, seed=1, allow_sleep=False), 200
    if cfg == 5:
        return scenes.config5(allow_sleep=False), 60
    raise ValueError(cfg)


def gpu_rate(sc, steps: int, solver: str, threads: int) -> dict:
    import torch

    from box2dpp_gb300.world import World

    w = World(sc)
    w.set_solver(solver)
    stream = torch.cuda.Stream()
    w.set_stream(stream.cuda_stream)
    w.upload()
    w.set_launch_plan([[0, 1, threads, 640, 1024]])
    # every step replayed from the captured graph (as the benchmark steps), timed in blocks of 50
    # steps between CUDA events on the handle's stream
    ms = []
    done = 0
    while done < steps:
        k = min(50, steps - done)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(k):
            w.graph_step(DT, VI, PI)
        b.record(stream)
        b.synchronize()
        ms.extend([a.elapsed_time(b) / k] * k)
        done += k
    w.sync()
    n = w.dynamic_bodies
    w.close()
    return {"solver": solver, "threads": threads, "steps": steps, "ms_per_step_mean": float(np.mean(ms)),
            "ms_per_step_median": float(np.median(ms)), "body_steps_per_s": n * steps / (sum(ms) / 1e3)}


def cpu_rate(sc, steps: int, budget_s: float) -> dict:
    import oracle

    w = oracle.OracleWorld(sc, "port", "libm")
    n = sum(1 for b in sc.bodies if b[0] == 2)
    done, t0 = 0, time.perf_counter()
    while done < steps and time.perf_counter() - t0 < budget_s:
        w.step(DT, VI, PI)
        done += 1
    el = time.perf_counter() - t0
    return {"cores": 1, "kind": "port", "steps": done, "seconds": round(el, 2), "body_steps_per_s": n * done / el,
            "sample": f"steps 1..{done} of the same scene on one thread"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--configs", default="1,2,5")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--threads", default="128,256,512", help="CTA widths to time")
    a = ap.parse_args()
    widths = [int(t) for t in a.threads.split(",")]
    for cfg in [int(c) for c in a.configs.split(",")]:
        sc, steps = scene(cfg)
        n = sum(1 for b in sc.bodies if b[0] == 2)
        line = {"config": cfg, "dynamic_bodies": n, "joints": len(sc.joints), "sleep": bool(sc.allow_sleep),
                "gpu": [gpu_rate(sc, steps, s, t) for s in ("plain", "coloured") for t in widths],
                "cpu": cpu_rate(sc, steps, a.cpu_seconds)}
        print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
