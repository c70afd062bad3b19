"""Benchmark of the GB300 Box2D step on the batched-worlds workload.

One step = one b2World::Step of every world of the batch: 4096 independent worlds (per GPU) whose
body counts are log-uniform in [16, 512], each a seeded pyramid, box stacks or a circle/polygon drop,
dt 1/60, float32, sleeping disabled (every body is simulated on every step). Metric: body-steps per
second (dynamic bodies x steps / time) over the whole job, at a stated velocity residual.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference] [--worlds n]

value: the batched step as shipped for throughput: the graph-coloured island solver (8/3 iterations
unless --coloured-vi says otherwise), launch plan picked by the online autotuner, each step replayed
from a captured CUDA graph; device time of the K timed steps (CUDA events on the stream the step
runs on), state resident in HBM (several hundred MB, larger than L2, so no flush between steps).
plain: the same measurement with the reference-order solver (bit-exact with the reference).
residual: the velocity residual (m/s, median over worlds of the last timed step) each solver leaves.
e2e: the same K coloured steps through the C-ABI with host buffers: every step uploads the force
and torque of every body from pinned host memory (gb_set_forces), steps (gb_world_graph_step) and
reads every body transform back into pinned host memory (gb_get_transforms), wall-clock timed.
--impl reference: the reference CPU step (the compiled reference where its build exists, else the
project's CPU restatement of it) on all host cores over the same worlds.
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

DT, VI, PI = 1.0 / 60.0, 8, 3
METRIC = "body-steps/sec at fixed residual (batched worlds)"
UNIT = "body-steps/s"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=60)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--worlds", type=int, default=4096)
    p.add_argument("--seed", type=int, default=1)
    p.add_argument("--cpu-steps", type=int, default=200, help="steps of the CPU baseline sample")
    p.add_argument("--coloured-vi", type=int, default=8, help="velocity iterations of the coloured solver")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-plain", action="store_true")
    return p.parse_args()


def dist_env():
    from box2dpp_gb300 import shard

    return shard.dist_env()


def workload(args, rank: int):
    """This rank's shard: its own args.worlds worlds (weak scaling, no data-path collective)."""
    from box2dpp_gb300 import shard

    return shard.shard_workload(args.worlds, args.seed, rank, allow_sleep=False)


def config_dict(args, worlds, extra=None):
    n = sum(w.dynamic_count for w in worlds)
    d = {
        "workload": f"batched: {len(worlds)} independent worlds per GPU, bodies log-uniform in [16,512] "
                    "(pyramid / box stacks / circle+polygon drop), dt 1/60, 8/3 iterations, sleep off",
        "worlds_per_gpu": len(worlds),
        "dynamic_bodies_per_gpu": n,
        "step": "one b2World::Step of every world",
        "l2": "state resident in HBM is larger than the 129 MB L2; no flush between steps",
        "parallelism": "independent worlds sharded across GPUs, no collective",
    }
    if extra:
        d.update(extra)
    return d


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        self.proc = None
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons), "samples": len(sm)}


# steps timed stage by stage after the timed region (gb_world_stage_times)
STAGE_STEPS = 5
STAGE_KERNELS = ["b2g::NarrowphaseKernel", "b2g::StepKernel", "b2g::ToiKernel", "b2g::StepToiKernel"]


def launches_per_step(n_classes: int) -> int:
    """Kernel launches of one step: each class of the launch plan is a pipeline of NarrowphaseKernel
    and ToiKernel (over that class's worlds' rows), StepKernel and StepToiKernel."""
    return 4 * n_classes


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


# DRAM bytes (read + write) per algorithmic byte of StepKernel (coloured solver), from one full ncu
# capture of the 1024-world case of this workload (111.0 MB read + 80.6 MB written for 41.4 MB
# algorithmic); traffic grows with the units processed, so the full launch's traffic is this ratio x
# its algorithmic bytes.
TRAFFIC_PER_ALGORITHMIC_BYTE = 191.6 / 41.4


def algorithmic_bytes(t: dict) -> int:
    """Minimum HBM bytes of one step if every persistent element is read and written once:
    104 B per solved body (52 B read: c, a, v, w, invMass, invI, localCenter, gravityScale, damping;
    24 B written c, a, v, w; 16 B transform; 12 B sweep c0, a0), 144 B per solved contact (manifold
    64 B read + 64 B written, body/fixture indices 8 B, friction/restitution 8 B), 32 B per proxy
    (fat AABB read + write), 8 B per broadphase pair."""
    return 104 * t["solved_bodies"] + 144 * t["solved_contacts"] + 32 * t["proxies"] + 8 * t["pairs"]


def cpu_baseline(worlds, steps: int, warmup: int, threads: int):
    """The reference CPU step (plain solver order) on `threads` host threads over all the worlds."""
    import oracle

    sample = worlds
    kind = "reference" if oracle.reference_available() and os.path.exists(os.path.join(ROOT, "oracle", "_ref",
                                                                                      "libref_libm.so")) else "port"
    trig = "libm" if kind == "reference" else "project"
    ws = [oracle.OracleWorld(s, kind, trig) for s in sample]
    # costliest first so the round-robin split over threads balances
    order = sorted(range(len(ws)), key=lambda i: -sample[i].dynamic_count)
    ws = [ws[i] for i in order]
    bodies = sum(s.dynamic_count for s in sample)
    oracle.step_many(ws, warmup, threads, DT, VI, PI)
    t0 = time.perf_counter()
    oracle.step_many(ws, steps, threads, DT, VI, PI)
    el = time.perf_counter() - t0
    return {
        "value": bodies * steps / el,
        "ms_per_step": el * 1e3 / max(steps, 1),
        "unit": UNIT,
        "cores": threads,
        "kind": kind,
        "sample": f"all {len(sample)} worlds ({bodies} dynamic bodies), {steps} steps after {warmup} warm-up "
                  f"steps, {el:.2f} s, 8/3 iterations (the reference's solver order)",
    }


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    worlds = workload(args, 0)
    threads = os.cpu_count() or 1
    cb = cpu_baseline(worlds, args.steps, args.warmup, threads)
    line = {
        "impl": "reference", "metric": METRIC, "value": cb["value"], "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": cb["ms_per_step"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": config_dict(args, worlds, {"sample": cb["sample"]}),
        "cpu_baseline": cb,
        "e2e": {"value": cb["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def _timed_steps(w, stream, steps: int, vi: int, clk=None):
    """K graph-replayed steps between two CUDA events on the step's stream; returns ms."""
    import torch

    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    start.record(stream)
    for _ in range(steps):
        w.graph_step(DT, vi, PI)
    end.record(stream)
    end.synchronize()
    return start.elapsed_time(end)


def _prepare(worlds, stream, solver: str, vi: int, warmup: int):
    """World batch on the GPU with the given solver, autotuned launch plan and warm-up steps."""
    from box2dpp_gb300.world import World

    w = World(worlds)
    w.set_stream(stream.cuda_stream)
    w.set_solver(solver, measure_residual=True)
    w.upload()
    w.autotune(2)
    tune_steps = 0
    while len(w.launch_plan()[1]) == 0 and tune_steps < 256:
        w.step(DT, vi, PI)
        tune_steps += 1
    for _ in range(warmup):
        w.graph_step(DT, vi, PI)
    w.sync()
    return w, tune_steps


def run_gpu(args):
    import numpy as np
    import torch

    rank, world_size, local = dist_env()
    torch.cuda.set_device(local)
    if world_size > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    worlds = workload(args, rank)
    stream = torch.cuda.Stream()

    def barrier():
        torch.cuda.synchronize()
        if world_size > 1:
            import torch.distributed as dist

            dist.barrier()
            torch.cuda.synchronize()

    def max_over_ranks(x: float) -> float:
        from box2dpp_gb300 import shard

        return shard.max_over_ranks(x, world_size, device="cuda")

    vi = args.coloured_vi
    w, tune_steps = _prepare(worlds, stream, "coloured", vi, args.warmup)
    n_dyn = w.dynamic_bodies
    t_before = w.totals()
    plan, cand_ms = w.launch_plan()
    barrier()
    with ClockSampler(local) as clk:
        ms = _timed_steps(w, stream, args.steps, vi)
    barrier()
    w.sync()
    t_after = w.totals()
    _, _, res = w.solver_stats()
    # per-stage device times of a few more steps (CUDA events between the step's launch stages), with
    # the same steps' work counts for the roofline of the stage that carries the step's state traffic
    stage_ms = np.zeros(4)
    stage_bytes = []
    for _ in range(STAGE_STEPS):
        stage_ms += w.stage_times(DT, vi, PI)
        stage_bytes.append(algorithmic_bytes(w.totals()))
    stage_ms /= STAGE_STEPS
    ms_max = max_over_ranks(ms)
    total_bodies = n_dyn * world_size
    value = total_bodies * args.steps / (ms_max / 1e3)

    # end-to-end through the C-ABI with pinned host buffers, over the same steps of the simulation as
    # the device-timed run (the scenes get denser as bodies settle, so later steps cost more): a
    # second handle on the same worlds with the chosen plan, replayed to the same step first (every
    # plan computes the same bits)
    nb = w.total_bodies
    w.close()
    from box2dpp_gb300.world import World

    we = World(worlds)
    we.set_stream(stream.cuda_stream)
    we.set_solver("coloured", measure_residual=True)
    we.upload()
    we.set_launch_plan(plan)
    for _ in range(tune_steps):
        we.step(DT, vi, PI)
    for _ in range(args.warmup):
        we.graph_step(DT, vi, PI)
    we.sync()
    forces = torch.zeros((nb, 4), dtype=torch.float32).pin_memory()
    xforms = torch.zeros((nb, 4), dtype=torch.float32).pin_memory()
    barrier()
    with clk:
        t0 = time.perf_counter()
        for _ in range(args.steps):
            we.set_forces_ptr(forces.data_ptr())
            we.graph_step(DT, vi, PI)
            we.get_transforms_ptr(xforms.data_ptr())
        we.sync()
        e2e_s = max_over_ranks(time.perf_counter() - t0)
    e2e_value = total_bodies * args.steps / e2e_s
    we.close()

    plain = None
    if not args.no_plain:
        wp, _ = _prepare(worlds, stream, "plain", VI, args.warmup)
        barrier()
        with clk:
            ms_p = max_over_ranks(_timed_steps(wp, stream, args.steps, VI))
        _, _, res_p = wp.solver_stats()
        plain_plan, _ = wp.launch_plan()
        plain = {"value": total_bodies * args.steps / (ms_p / 1e3), "unit": UNIT, "ms_per_step": ms_p / args.steps,
                 "velocity_iterations": VI, "residual_median": float(np.median(res_p)),
                 "launch_plan": plain_plan.tolist(),
                 "note": "reference-order per-island Gauss-Seidel, bit-exact with the reference"}
        wp.close()

    if rank == 0:
        peak, peak_kind = measured_peaks()
        step_bytes = float(np.mean(stage_bytes))
        kernel_ms = float(stage_ms[1])
        achieved = step_bytes / (kernel_ms / 1e3) / 1e9
        total_stage = float(stage_ms.sum())
        roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": step_bytes * TRAFFIC_PER_ALGORITHMIC_BYTE, "peak_source": peak_kind,
                "traffic_note": "DRAM bytes per launch stage, scaled from an ncu capture of StepKernel on the "
                                "1024-world case (traffic per algorithmic byte)",
                "kernel": "b2g::StepKernel",
                "algorithmic_bytes_per_launch": step_bytes,
                "launch_ms": kernel_ms,
                "note": "StepKernel's stage (every class of the plan) carries the step's persistent-state "
                        "traffic (collide commit, island solve, fixture sync, pair finding); its bytes per "
                        f"step over its CUDA-event duration, averaged over {STAGE_STEPS} steps after the timed "
                        "region",
                "stages": {k: {"ms": float(m), "share": float(m) / total_stage}
                           for k, m in zip(STAGE_KERNELS, stage_ms)},
                "counts_per_step": {k: (t_before[k] + t_after[k]) / 2.0 for k in
                                    ("solved_bodies", "solved_contacts", "proxies", "pairs", "toi_events")}}
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world_size, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": config_dict(args, worlds, {
                "solver": f"graph-coloured, {vi}/3 iterations",
                "launch_plan": plan.tolist(), "autotune_candidate_ms": [round(float(x), 3) for x in cand_ms],
                "autotune_steps": tune_steps, "cuda_graph": "one captured step replayed per step"}),
            "residual": {"coloured_median": float(np.median(res)), "unit": "m/s",
                         "definition": "max over contact points of the natural-map residual in m/s: |vn - bias| on "
                                       "active normal points, |vt| on friction inside its cone, 0 at a solution; "
                                       "after the velocity iterations"},
            "plain": plain,
            "roofline": roof,
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": nb * 16, "d2h_bytes_per_step": nb * 16,
                    "calls": "gb_set_forces + gb_world_graph_step + gb_get_transforms per step, pinned host buffers"},
            "gpu_launches": args.steps * launches_per_step(len(plan)),
            "clocks": clk.summary(),
        }
        if not args.no_cpu_baseline and world_size == 1:
            line["cpu_baseline"] = cpu_baseline(worlds, args.cpu_steps, args.warmup, os.cpu_count() or 1)
        print(json.dumps(line), flush=True)
    if world_size > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
