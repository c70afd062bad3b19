"""Train the learned warm start and measure what it saves.

  python -m box2dpp_gb300.train_warmstart [--seeds 16] [--bodies 10000] [--steps 20000] [--batch 65536] [--out PATH]

1. Data: worlds of the config-2 mix (circles and convex polygons dropped into an edge container,
   ``scenes.config4``), one per seed over ``--seeds`` held-out seeds, stepped with the plain
   (reference-order) solver. After ``--settle`` steps at 8/3 iterations the contact-point log records,
   for ``--log-steps`` steps at ``--log-vi`` velocity iterations, each island contact point's 14
   features at the start of the velocity solve and the impulses the iterations end with (in velocity
   units); the network learns the difference between those and the reference warm start.
2. Training: the library's tensor-core kernels, Adam for ``--steps`` steps on batches of ``--batch``
   points drawn from the log: the points the reference warm start leaves cold (``--points cold``, the
   network then predicts only those), or every point (``--points all``, the network corrects every
   point's reference warm start).
3. Evaluation on other seeds: first the plain solver with the reference warm start at 8 velocity
   iterations gives the residual the reference reaches (the median over the evaluation worlds and
   steps: the benchmark's matched accuracy); then the plain solver with that residual as its
   tolerance (at most ``--max-vi`` iterations) counts the iterations per island contact it needs
   with the reference warm start and with the learned one (which falls back to the reference warm
   start whenever its residual is worse). ``--tol`` > 0 replaces the measured target.

The trained parameters and normaliser are written to ``--out`` (``box2dpp_gb300/data/warmstart_mlp.npz``
by default) together with the evaluation numbers.
"""
from __future__ import annotations

import argparse
import json
import os
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
DEFAULT_OUT = os.path.join(HERE, "data", "warmstart_mlp.npz")
DT, PI = 1.0 / 60.0, 3


def log_points(first_seed: int, n_seeds: int, bodies: int, settle: int, log_steps: int, log_vi: int,
               chunk: int = 250):
    from . import scenes
    from .world import World

    xs, ts = [], []
    for s0 in range(first_seed, first_seed + n_seeds, chunk):
        n = min(chunk, first_seed + n_seeds - s0)
        w = World(scenes.config4(n, s0, bodies))
        w.set_solver("plain")
        for _ in range(settle):
            w.step(DT, 8, PI)
        w.set_contact_log(4_000_000)
        for _ in range(log_steps):
            w.step(DT, log_vi, PI)
            x, t = w.read_contact_log()
            xs.append(x)
            ts.append(t)
        w.close()
    return np.concatenate(xs), np.concatenate(ts)


def correction_targets(x: np.ndarray, t: np.ndarray) -> np.ndarray:
    """The network's targets: the logged final impulses minus the reference warm start (features 9
    and 10), both in velocity units."""
    return (t - x[:, 9:11]).astype(np.float32)


def cold_points(x: np.ndarray, t: np.ndarray):
    """The logged points the reference warm start leaves cold (no normal impulse carried over): the
    only points the step lets the network predict."""
    keep = ~(x[:, 9] > 0.0)
    return x[keep], t[keep]


def iterations_to_tolerance(mlp, first_seed: int, n_seeds: int, bodies: int, settle: int, steps: int, tol: float,
                            max_vi: int, all_points: bool = False):
    """Mean velocity iterations per island contact the plain solver runs to reach tol (at most
    max_vi), the share of islands that kept the learned prediction (None without a network) and the
    median residual the iterations end with."""
    from . import scenes
    from .world import World

    w = World(scenes.config4(n_seeds, first_seed, bodies))
    w.set_solver("plain", tolerance=tol, measure_residual=True)
    for _ in range(settle):
        w.step(DT, 8, PI)
    w.set_warm_start(mlp, all_points)
    its = contacts = isl = kept = 0
    res = []
    for _ in range(steps):
        w.step(DT, max_vi, PI)
        used, it_sum = w.warm_stats()
        its += int(it_sum.sum())
        contacts += int(w.totals()["solved_contacts"])
        isl += sum(w.stats(i)[0] for i in range(w.n_worlds))
        kept += int(used.sum())
        res.append(w.solver_stats()[2].copy())
    w.close()
    return its / max(contacts, 1), (kept / max(isl, 1) if mlp is not None else None), float(np.median(np.array(res)))


def reference_residual(first_seed: int, n_seeds: int, bodies: int, settle: int, steps: int, vi: int = 8) -> float:
    """Median velocity residual (m/s) the plain solver with the reference warm start leaves after vi
    iterations, over the worlds and the steps after settling."""
    from . import scenes
    from .world import World

    w = World(scenes.config4(n_seeds, first_seed, bodies))
    w.set_solver("plain", measure_residual=True)
    for _ in range(settle):
        w.step(DT, 8, PI)
    res = []
    for _ in range(steps):
        w.step(DT, vi, PI)
        res.append(w.solver_stats()[2].copy())
    w.close()
    return float(np.median(np.array(res)))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--seeds", type=int, default=16)
    ap.add_argument("--first-seed", type=int, default=1_000_000)
    ap.add_argument("--bodies", type=int, default=10000)
    ap.add_argument("--settle", type=int, default=60)
    ap.add_argument("--log-steps", type=int, default=8)
    ap.add_argument("--log-vi", type=int, default=40)
    ap.add_argument("--steps", type=int, default=20000)
    ap.add_argument("--batch", type=int, default=65536)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--eval-seeds", type=int, default=4)
    ap.add_argument("--eval-first-seed", type=int, default=2_000_000)
    ap.add_argument("--eval-steps", type=int, default=30)
    ap.add_argument("--tol", type=float, default=0.0, help="> 0: this target instead of the measured one")
    ap.add_argument("--max-vi", type=int, default=64)
    ap.add_argument("--points", default="all", choices=["cold", "all"],
                    help="train on (and predict) the cold points only, or every point")
    ap.add_argument("--out", default=DEFAULT_OUT)
    args = ap.parse_args()

    from .learn import Mlp

    t0 = time.time()
    x, t = log_points(args.first_seed, args.seeds, args.bodies, args.settle, args.log_steps, args.log_vi)
    t_log = time.time() - t0
    n_logged = len(x)
    all_points = args.points == "all"
    if not all_points:
        x, t = cold_points(x, t)
    m = Mlp(1)
    m.fit_normaliser(x)
    t0 = time.time()
    losses = m.train(x, correction_targets(x, t), steps=args.steps, batch=args.batch, lr=args.lr, seed=1)
    t_train = time.time() - t0
    target = args.tol if args.tol > 0 else reference_residual(args.eval_first_seed, args.eval_seeds, args.bodies,
                                                              args.settle, args.eval_steps)
    ref_its, _, ref_res = iterations_to_tolerance(None, args.eval_first_seed, args.eval_seeds, args.bodies,
                                                  args.settle, args.eval_steps, target, args.max_vi)
    lrn_its, used, lrn_res = iterations_to_tolerance(m, args.eval_first_seed, args.eval_seeds, args.bodies,
                                                     args.settle, args.eval_steps, target, args.max_vi, all_points)
    report = {
        "points_logged": int(n_logged), "points_trained": int(len(x)), "points": args.points, "log_seconds": round(t_log, 1), "train_steps": args.steps, "batch": args.batch,
        "train_seconds": round(t_train, 1), "loss_first": float(losses[:10].mean()),
        "loss_last": float(losses[-100:].mean()), "tolerance": target,
        "tolerance_rule": "given" if args.tol > 0 else "median residual of the reference warm start after 8 iterations",
        "bodies_per_world": args.bodies, "max_vi": args.max_vi,
        "iterations_reference": ref_its, "iterations_learned": lrn_its, "ratio": lrn_its / ref_its,
        "learned_kept_share": used, "residual_median_reference": ref_res, "residual_median_learned": lrn_res,
        "train_seeds": [args.first_seed, args.first_seed + args.seeds - 1],
        "eval_seeds": [args.eval_first_seed, args.eval_first_seed + args.eval_seeds - 1],
    }
    os.makedirs(os.path.dirname(os.path.abspath(args.out)), exist_ok=True)
    p, mu, sigma = m.params()
    np.savez(args.out, params=p, mu=mu, sigma=sigma, report=json.dumps(report))
    print(json.dumps(report), flush=True)


if __name__ == "__main__":
    main()
