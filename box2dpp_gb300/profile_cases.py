"""Small, self-contained workloads for profiling the library's kernels (ncu) and for quick timing.

  python -m box2dpp_gb300.profile_cases step [--worlds 1024] [--solver coloured|plain] [--steps 6]
  python -m box2dpp_gb300.profile_cases mlp [--rows 262144] [--batch 65536] [--steps 20]

``step`` builds the batched-worlds workload (log-uniform [16, 512] bodies per world; pyramids, box
stacks, circle/polygon drops; sleep off) and runs ``--steps`` steps with the default launch plan
(one StepKernel launch per step). ``mlp`` trains the learned warm start's network on seeded
synthetic rows (one MlpTrainKernel and one Adam launch per step). Both exit 0 and print one line.
"""
from __future__ import annotations

import argparse
import sys


def run_step(worlds: int, solver: str, steps: int) -> str:
    from . import scenes
    from .world import World

    w = World(scenes.config3(worlds, seed=1, allow_sleep=False))
    w.set_solver(solver)
    for _ in range(steps):
        w.step()
    w.sync()
    return f"step ok {w.totals()}"


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
    m = sub.add_parser("mlp")
    m.add_argument("--rows", type=int, default=262144)
    m.add_argument("--batch", type=int, default=65536)
    m.add_argument("--steps", type=int, default=20)
    a = ap.parse_args(argv)
    print(run_step(a.worlds, a.solver, a.steps) if a.case == "step" else run_mlp(a.rows, a.batch, a.steps), flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
