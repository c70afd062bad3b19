"""Small, self-contained workloads for profiling the library's kernels (ncu) and for quick timing.

  python -m box2dpp_gb300.profile_cases step [--worlds 1024] [--solver coloured|plain] [--steps 6] [--vi 8] [--autotune]
  python -m box2dpp_gb300.profile_cases mlp [--rows 262144] [--batch 65536] [--steps 20]

``step`` builds the benchmark's batched-worlds workload (its first ``--worlds`` worlds: log-uniform
[16, 512] bodies per world; pyramids, box stacks, circle/polygon drops; sleep off) and runs
``--steps`` steps with the default launch plan (one StepKernel launch per step), or with
``--autotune`` the autotuner's trials (12 candidate plans, one step each) and then its pick. ``mlp`` trains the learned warm start's network on seeded
synthetic rows (one MlpTrainKernel and one Adam launch per step). Both exit 0 and print one line.
"""
from __future__ import annotations

import argparse
import sys


def run_step(worlds: int, solver: str, steps: int, vi: int = 8, autotune: bool = False) -> str:
    from . import shard
    from .world import World

    # the benchmark's worlds (shard 0 of its workload)
    w = World(shard.shard_workload(worlds, 1, 0, allow_sleep=False))
    w.set_solver(solver)
    w.upload()
    if autotune:
        w.autotune(1)
    for _ in range(steps):
        w.step(1.0 / 60.0, vi, 3)
    w.sync()
    return f"step ok plan {w.launch_plan()[0].tolist()} {w.totals()}"


def run_mlp(rows: int, batch: int, steps: int) -> str:
    import numpy as np

    from .learn import Mlp

    rng = np.random.default_rng(0)
    x = rng.normal(0, 1, (rows, 14)).astype(np.float32)
    t = rng.normal(0, 1, (rows, 2)).astype(np.float32)
    m = Mlp(1)
    m.fit_normaliser(x)
    losses = m.train(x, t, steps=steps, batch=batch, lr=1e-3)
    return f"mlp ok last loss {float(losses[-1]):.4f}"


def main(argv=None) -> int:
    ap = argparse.ArgumentParser()
    sub = ap.add_subparsers(dest="case", required=True)
    s = sub.add_parser("step")
    s.add_argument("--worlds", type=int, default=1024)
    s.add_argument("--solver", default="coloured", choices=["coloured", "plain"])
    s.add_argument("--steps", type=int, default=6)
    s.add_argument("--vi", type=int, default=8, help="velocity iterations")
    s.add_argument("--autotune", action="store_true", help="arm the launch-plan autotuner first")
    m = sub.add_parser("mlp")
    m.add_argument("--rows", type=int, default=262144)
    m.add_argument("--batch", type=int, default=65536)
    m.add_argument("--steps", type=int, default=20)
    a = ap.parse_args(argv)
    print(run_step(a.worlds, a.solver, a.steps, a.vi, a.autotune) if a.case == "step"
          else run_mlp(a.rows, a.batch, a.steps), flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
