"""Report on the joint stress world (``scenes.config5``): step time, energy drift and penetration
with the plain (reference-order) and the graph-coloured solver.

  python -m box2dpp_gb300.stress [--bodies 65536] [--chains 512] [--steps 120] [--solvers plain,coloured]

Mechanical energy is summed over the dynamic bodies (kinetic, translational and rotational, plus
potential m g y) from their shapes' mass data; the world is not conservative (the container turns,
contacts are inelastic and frictional), so the drift is reported as a diagnostic, in % of the
initial energy per simulated second. Penetration is the deepest contact penetration the position
solver starts from in each step (gb_world_contact_stats).
"""
from __future__ import annotations

import argparse
import json
import math
import time

import numpy as np

DT = 1.0 / 60.0


def mass_data(scene):
    """(mass, rotational inertia about the centre) per body from its box/circle fixtures."""
    nb = len(scene.bodies)
    m = np.zeros(nb)
    inertia = np.zeros(nb)
    for body, type_, shape, n, mat, _ in scene.fixtures:
        rho = mat[0]
        if type_ == 3:  # box (half extents, centred)
            hx, hy = shape[0], shape[1]
            mm = 4.0 * hx * hy * rho
            m[body] += mm
            inertia[body] += mm * (hx * hx + hy * hy) / 3.0
        elif type_ == 0:  # circle
            r = shape[2]
            mm = math.pi * r * r * rho
            m[body] += mm
            inertia[body] += mm * (0.5 * r * r + shape[0] ** 2 + shape[1] ** 2)
    return m, inertia


def energy(bodies, m, inertia, dynamic, g=10.0):
    v2 = bodies[:, 5] ** 2 + bodies[:, 6] ** 2
    e = 0.5 * m * v2 + 0.5 * inertia * bodies[:, 7] ** 2 + m * g * bodies[:, 4]
    return float(e[dynamic].sum())


def run(solver: str, n_bodies: int, n_chains: int, steps: int, half: float) -> dict:
    import torch

    from . import scenes
    from .world import World

    sc = scenes.config5(n_bodies=n_bodies, n_chains=n_chains, half=half)
    m, inertia = mass_data(sc)
    dynamic = np.array([b[0] == scenes.DYNAMIC for b in sc.bodies])
    w = World(sc)
    w.set_solver(solver, measure_residual=True)
    stream = torch.cuda.Stream()
    w.set_stream(stream.cuda_stream)
    w.upload()
    e0 = energy(w.bodies(0), m, inertia, dynamic)
    pen, ms = [], []
    for _ in range(steps):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        w.step(DT, 8, 3)
        b.record(stream)
        b.synchronize()
        ms.append(a.elapsed_time(b))
        pen.append(float(w.max_penetration()[0]))
    bodies = w.bodies(0)
    e1 = energy(bodies, m, inertia, dynamic)
    res = float(w.solver_stats()[2][0])
    w.sync()
    w.close()
    secs = steps * DT
    return {
        "solver": solver, "bodies": int(dynamic.sum()), "joints": len(sc.joints), "steps": steps,
        "ms_per_step_median": float(np.median(ms)), "ms_per_step_first": float(ms[0]),
        "body_steps_per_s": float(dynamic.sum()) * steps / (sum(ms) / 1e3),
        "energy_initial": e0, "energy_final": e1, "energy_drift_pct_per_s": 100.0 * (e1 - e0) / abs(e0) / secs,
        "max_penetration_m": max(pen), "penetration_last_m": pen[-1], "velocity_residual_last": res,
        "finite": bool(np.all(np.isfinite(bodies))),
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--bodies", type=int, default=65536)
    ap.add_argument("--chains", type=int, default=512)
    ap.add_argument("--half", type=float, default=150.0)
    ap.add_argument("--steps", type=int, default=120)
    ap.add_argument("--solvers", default="coloured,plain")
    a = ap.parse_args()
    for solver in a.solvers.split(","):
        t0 = time.time()
        r = run(solver, a.bodies, a.chains, a.steps, a.half)
        r["wall_s"] = round(time.time() - t0, 1)
        print(json.dumps(r), flush=True)


if __name__ == "__main__":
    main()
