"""Benchmark of the GB300 Box2D step on the batched-worlds workload.

One step = one b2World::Step of every world of the batch: 4096 independent worlds (per GPU) whose
body counts are log-uniform in [16, 512], each a seeded pyramid, box stacks or a circle/polygon drop,
dt 1/60, float32, sleeping disabled (every body is simulated on every step). Metric: body-steps per
second (dynamic bodies x steps / time) over the whole job, at a matched velocity residual.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference] [--worlds n]

Every arm runs the same simulation steps: PRE_STEPS steps (the launch-plan autotuner's trials on
the GPU), W warm-up steps, then the K timed steps.
arms.plain: the reference-order solver (bit-exact with the reference), 8/3 iterations; its median
velocity residual (measured on the step after the timed window, which the timed steps do not spend
time on) is the accuracy every other arm must reach.
arms.coloured: the graph-coloured island solver at the fewest velocity iterations (of COLOURED_VI)
whose median residual is no larger than plain's (coloured_search lists each try).
arms.learned: the reference-order solver with the learned warm start (a network trained first by the
library's kernels on the plain solver's converged impulses, logged from held-out worlds of the same
workload), at the fewest velocity iterations (of LEARNED_VI) whose median residual is no larger than
plain's (learned_search lists each try; no arm when none qualifies).
value: the faster of those arms (headline names it): device time of the K timed steps, each step
replayed from a captured CUDA graph, CUDA events on the stream the step runs on, state resident in
HBM (several hundred MB, larger than L2, so no flush between steps).
e2e: the headline arm's same K steps through the C-ABI with host buffers: every step uploads the
force and torque of every body from pinned host memory (gb_set_forces_async), steps
(gb_world_graph_step) and reads every body transform back into pinned host memory
(gb_get_transforms_async); the copies run on their own streams and overlap the neighbouring steps,
and gb_world_sync after the last step waits for every copy; wall-clock timed; each arm carries its
own e2e figure.
sleep_on: the headline arm with sleeping allowed (the reference's default), beside the CPU figure.
--impl reference: the reference CPU step (the compiled reference where its build exists, else the
project's CPU restatement of it, bit-exact with it) with glibc trig on all host cores over the same
worlds and the same steps.
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
# Steps every arm runs before its warm-up and timed window: the launch-plan autotuner's trials (12
# candidate plans x 2 steps each on the bench batch). The CPU arms advance the same steps untimed.
PRE_STEPS = 24
# velocity iterations tried for the graph-coloured solver, fewest first, until its median residual
# matches the reference-order solver's
COLOURED_VI = (8, 9, 10, 11, 12, 14, 16, 20, 24, 32)
# velocity iterations tried for the reference-order solver with the learned warm start
LEARNED_VI = (4, 5, 6, 7, 8)
# the learned warm start's training: held-out worlds (seed offset), logged steps, Adam steps
LEARN_SEED_OFFSET, LEARN_WORLDS, LEARN_LOG_STEPS, LEARN_LOG_VI, LEARN_TRAIN_STEPS, LEARN_BATCH = 1000, 512, 8, 40, 3000, 16384
METRIC = "body-steps/sec at fixed residual (batched worlds)"
UNIT = "body-steps/s"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--worlds", type=int, default=4096)
    p.add_argument("--seed", type=int, default=1)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-coloured", action="store_true", help="measure the reference-order solver only")
    p.add_argument("--no-sleep-on", action="store_true", help="skip the sleep-on line")
    p.add_argument("--no-learned", action="store_true", help="skip the learned warm-start arm")
    return p.parse_args()


def dist_env():
    from box2dpp_gb300 import shard

    return shard.dist_env()


def workload(args, rank: int, allow_sleep: bool = False):
    """This rank's shard: its part, by estimated cost, of the job's args.worlds worlds per rank (weak
    scaling, no data-path collective)."""
    from box2dpp_gb300 import shard

    _, world_size, _ = dist_env()
    return shard.shard_workload(args.worlds, args.seed, rank, allow_sleep=allow_sleep, world_size=world_size)


def config_dict(args, worlds):
    """The workload, identical for both arms (the GPU arm's solver details are reported beside it)."""
    n = sum(w.dynamic_count for w in worlds)
    first = PRE_STEPS + args.warmup + 1
    return {
        "workload": f"batched: {len(worlds)} independent worlds per GPU, bodies log-uniform in [16,512] "
                    "(pyramid / box stacks / circle+polygon drop), dt 1/60, sleep off",
        "worlds_per_gpu": len(worlds),
        "dynamic_bodies_per_gpu": n,
        "step": "one b2World::Step of every world",
        "timed_steps": f"{first}-{first + args.steps - 1}",
        "accuracy": "matched: median velocity residual no larger than the reference-order solver's at 8/3 "
                    "iterations",
        "l2": "state resident in HBM is larger than the 129 MB L2; no flush between steps",
        "parallelism": "one world set partitioned across GPUs by body count, no collective",
    }


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


# DRAM bytes (read + write) per algorithmic byte of StepKernel, from a full ncu capture per solver of
# one step of the 1024-world case of this workload (coloured, all four classes of the tuned plan:
# 84.5 MB read + 17.1 MB written for 42.0 MB algorithmic; plain, default plan: 114.6 MB + 82.2 MB for
# 41.4 MB); traffic grows with the units processed, so the full launch's traffic is this ratio x its
# algorithmic bytes.
TRAFFIC_PER_ALGORITHMIC_BYTE = {"coloured": 101.6 / 42.0, "plain": 196.7 / 41.4}


def algorithmic_bytes(t: dict) -> int:
    """Minimum HBM bytes of one step if every persistent element is read and written once:
    104 B per solved body (52 B read: c, a, v, w, invMass, invI, localCenter, gravityScale, damping;
    24 B written c, a, v, w; 16 B transform; 12 B sweep c0, a0), 144 B per solved contact (manifold
    64 B read + 64 B written, body/fixture indices 8 B, friction/restitution 8 B), 32 B per proxy
    (fat AABB read + write), 8 B per broadphase pair."""
    return 104 * t["solved_bodies"] + 144 * t["solved_contacts"] + 32 * t["proxies"] + 8 * t["pairs"]


def cpu_baseline(worlds, steps: int, warmup: int, threads: int, sleep: bool = False):
    """The reference CPU step (the reference's solver order) on `threads` host threads over all the
    worlds, with glibc's sinf/cosf (the reference's own trig). The worlds first advance through the
    same steps the GPU arm spends before its timed window (PRE_STEPS tuning steps + `warmup`), so both
    arms time the same simulation steps."""
    import oracle

    kind = "reference" if oracle.reference_available() and os.path.exists(os.path.join(ROOT, "oracle", "_ref",
                                                                                      "libref_libm.so")) else "port"
    ws = [oracle.OracleWorld(s, kind, "libm") for s in worlds]
    # costliest first so the round-robin split over threads balances
    order = sorted(range(len(ws)), key=lambda i: -worlds[i].dynamic_count)
    ws = [ws[i] for i in order]
    bodies = sum(s.dynamic_count for s in worlds)
    oracle.step_many(ws, PRE_STEPS + warmup, threads, DT, VI, PI)
    t0 = time.perf_counter()
    oracle.step_many(ws, steps, threads, DT, VI, PI)
    el = time.perf_counter() - t0
    first = PRE_STEPS + warmup + 1
    return {
        "value": bodies * steps / el,
        "ms_per_step": el * 1e3 / max(steps, 1),
        "unit": UNIT,
        "cores": threads,
        "kind": kind,
        "trig": "glibc sinf/cosf",
        "sleep": "on" if sleep else "off",
        "sample": f"all {len(worlds)} worlds ({bodies} dynamic bodies), steps {first}-{first + steps - 1} "
                  f"(after the same {PRE_STEPS + warmup} steps the GPU arm runs before its timed window), "
                  f"{el:.2f} s, 8/3 iterations in the reference's solver order",
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
        "config": config_dict(args, worlds),
        "cpu_baseline": cb,
        "e2e": {"value": cb["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def _timed_steps(w, stream, steps: int, vi: int):
    """K graph-replayed steps between two CUDA events on the step's stream; returns ms."""
    import torch

    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    start.record(stream)
    for _ in range(steps):
        w.graph_step(DT, vi, PI)
    end.record(stream)
    end.synchronize()
    return start.elapsed_time(end)


def _prepare(worlds, stream, solver: str, vi: int, warmup: int, plan=None, mlp=None):
    """World batch on the GPU with the given solver (and learned warm start, with a network),
    advanced to the timed window: PRE_STEPS steps (the online autotuner picks the launch plan during
    them unless a plan is given) and `warmup` graph-replayed steps."""
    from box2dpp_gb300.world import World

    w = World(worlds)
    w.set_stream(stream.cuda_stream)
    w.set_solver(solver)
    w.upload()
    if mlp is not None:
        w.set_warm_start(mlp, all_points=True)
    if plan is None:
        w.autotune(2)
    else:
        w.set_launch_plan(plan)
    for _ in range(PRE_STEPS):
        w.step(DT, vi, PI)
    if plan is None and len(w.launch_plan()[1]) == 0:
        raise RuntimeError(f"the launch-plan autotuner needs more than {PRE_STEPS} steps")
    for _ in range(warmup):
        w.graph_step(DT, vi, PI)
    w.sync()
    return w


def train_learned(args):
    """The learned warm start's network, trained by the library's kernels: the plain solver's final
    impulses at LEARN_LOG_VI velocity iterations, logged for LEARN_LOG_STEPS steps after PRE_STEPS
    steps on LEARN_WORLDS held-out worlds of the workload (another seed), every logged point (the
    network corrects every point's warm start). Returns (network, points trained on, seconds)."""
    import numpy as np

    from box2dpp_gb300 import shard
    from box2dpp_gb300.learn import Mlp
    from box2dpp_gb300.train_warmstart import correction_targets
    from box2dpp_gb300.world import World

    t0 = time.perf_counter()
    w = World(shard.shard_workload(LEARN_WORLDS, args.seed + LEARN_SEED_OFFSET, 0))
    w.set_solver("plain")
    for _ in range(PRE_STEPS):
        w.step(DT, VI, PI)
    w.set_contact_log(1_000_000)
    xs, ts = [], []
    for _ in range(LEARN_LOG_STEPS):
        w.step(DT, LEARN_LOG_VI, PI)
        x, t = w.read_contact_log()
        xs.append(x.copy())
        ts.append(t.copy())
    w.close()
    x, t = np.concatenate(xs), np.concatenate(ts)
    m = Mlp(1)
    m.fit_normaliser(x)
    m.train(x, correction_targets(x, t), steps=LEARN_TRAIN_STEPS, batch=LEARN_BATCH, lr=1e-3, seed=1)
    return m, len(x), time.perf_counter() - t0


def _e2e(worlds, stream, solver: str, vi: int, plan, args, clk, max_over_ranks, barrier, mlp=None):
    """The same K steps end to end through the C-ABI with pinned host buffers: a handle on the same
    worlds with the given plan, advanced through the same steps, then per step gb_set_forces_async
    (every body's force and torque from pinned host memory), gb_world_graph_step and
    gb_get_transforms_async (every body's transform into pinned host memory; the copies of one step
    overlap the next step), and gb_world_sync after the last, wall-clock timed."""
    import torch

    we = _prepare(worlds, stream, solver, vi, args.warmup, plan, mlp)
    nb = we.total_bodies
    forces = torch.zeros((nb, 4), dtype=torch.float32).pin_memory()
    xforms = torch.zeros((nb, 4), dtype=torch.float32).pin_memory()
    barrier()
    with clk:
        t0 = time.perf_counter()
        for _ in range(args.steps):
            we.set_forces_async_ptr(forces.data_ptr())
            we.graph_step(DT, vi, PI)
            we.get_transforms_async_ptr(xforms.data_ptr())
        we.sync()
        e2e_s = max_over_ranks(time.perf_counter() - t0)
    we.close()
    return e2e_s, nb


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

    n_dyn = sum(s.dynamic_count for s in worlds)
    total_bodies = n_dyn * world_size
    clk = ClockSampler(local)

    def device_arm(solver: str, vi: int, plan=None, mlp=None):
        """K timed steps of one solver; (record, handle) with the handle kept for the stage times."""
        w = _prepare(worlds, stream, solver, vi, args.warmup, plan, mlp)
        t_before = w.totals()
        barrier()
        with clk:
            ms = max_over_ranks(_timed_steps(w, stream, args.steps, vi))
        barrier()
        w.sync()
        t_after = w.totals()
        # the accuracy of the arm: the velocity residual measured on the step after the timed window
        # (measuring it is a diagnostic, not part of b2World::Step, so the timed steps do not)
        w.set_solver(solver, measure_residual=True)
        w.graph_step(DT, vi, PI)
        w.sync()
        _, _, res = w.solver_stats()
        w.set_solver(solver)
        chosen, cand_ms = w.launch_plan()
        rec = {"solver": solver, "warm_start": "reference" if mlp is None else "learned", "velocity_iterations": vi,
               "value": total_bodies * args.steps / (ms / 1e3),
               "unit": UNIT, "ms_per_step": ms / args.steps, "residual_median": float(np.median(res)),
               "launch_plan": chosen.tolist(), "autotune_candidate_ms": [round(float(x), 3) for x in cand_ms],
               "counts_per_step": {k: (t_before[k] + t_after[k]) / 2.0 for k in
                                   ("solved_bodies", "solved_contacts", "proxies", "pairs", "toi_events")}}
        return rec, w

    # 1. the reference-order solver (bit-exact with the reference): its residual is the accuracy every
    #    other arm must match
    plain, wp = device_arm("plain", VI)
    arms = {"plain": (plain, wp)}
    # 2. the graph-coloured solver at the fewest velocity iterations whose median residual is no
    #    larger than the plain solver's (same simulation steps), launch plan tuned once at 8 iterations
    searched = []
    coloured_plan = None
    if not args.no_coloured:
        for vi in COLOURED_VI:
            rec, wc = device_arm("coloured", vi, coloured_plan)
            if coloured_plan is None:
                coloured_plan = np.asarray(rec["launch_plan"], dtype=np.int32)
            searched.append({"velocity_iterations": vi, "residual_median": rec["residual_median"],
                             "ms_per_step": rec["ms_per_step"]})
            if rec["residual_median"] <= plain["residual_median"]:
                arms["coloured"] = (rec, wc)
                break
            wc.close()
    # 3. the reference-order solver with the learned warm start at the fewest velocity iterations whose
    #    median residual is no larger than the plain solver's
    learned_search = []
    learned_info = None
    mlps = {}
    if not args.no_learned:
        mlp, n_points, train_s = train_learned(args)
        learned_info = {"points_trained": n_points, "seconds": round(train_s, 1), "train_steps": LEARN_TRAIN_STEPS,
                        "worlds": LEARN_WORLDS, "seed": args.seed + LEARN_SEED_OFFSET}
        plain_plan = np.asarray(plain["launch_plan"], dtype=np.int32)
        for vi in LEARNED_VI:
            rec, wl = device_arm("plain", vi, plain_plan, mlp)
            used, _ = wl.warm_stats()
            searched_rec = {"velocity_iterations": vi, "residual_median": rec["residual_median"],
                            "ms_per_step": rec["ms_per_step"], "islands_keeping_prediction": int(used.sum())}
            learned_search.append(searched_rec)
            if rec["residual_median"] <= plain["residual_median"]:
                arms["learned"] = (rec, wl)
                mlps["learned"] = mlp
                break
            wl.close()
    # the headline: the fastest arm at matched accuracy (plain always qualifies)
    head_name = max(arms, key=lambda k: arms[k][0]["value"])
    head, wh = arms[head_name]
    # per-stage device times of a few more steps of the headline arm (CUDA events between the step's
    # launch stages), with the same steps' work counts for the roofline of the stage that carries the
    # step's persistent-state traffic
    stage_ms = np.zeros(4)
    stage_bytes = []
    for _ in range(STAGE_STEPS):
        stage_ms += wh.stage_times(DT, head["velocity_iterations"], PI)
        stage_bytes.append(algorithmic_bytes(wh.totals()))
    stage_ms /= STAGE_STEPS
    for _, (_, h) in arms.items():
        h.close()
    # end to end through the C-ABI, for every arm
    for name, (rec, _) in arms.items():
        e2e_s, nb = _e2e(worlds, stream, rec["solver"], rec["velocity_iterations"],
                         np.asarray(rec["launch_plan"], dtype=np.int32), args, clk, max_over_ranks, barrier,
                         mlps.get(name))
        rec["e2e"] = {"value": total_bodies * args.steps / e2e_s, "unit": UNIT, "h2d_bytes_per_step": nb * 16,
                      "d2h_bytes_per_step": nb * 16,
                      "calls": "gb_set_forces_async + gb_world_graph_step + gb_get_transforms_async per step "
                               "(pinned host buffers, copies overlapping the next step), gb_world_sync after "
                               "the last"}
    # sleep on (the reference's default): the headline arm on the same worlds with sleeping allowed
    sleep_on = None
    if not args.no_sleep_on:
        worlds_sleep = workload(args, rank, allow_sleep=True)
        ws = _prepare(worlds_sleep, stream, head["solver"], head["velocity_iterations"], args.warmup,
                      np.asarray(head["launch_plan"], dtype=np.int32), mlps.get(head_name))
        barrier()
        with clk:
            ms_s = max_over_ranks(_timed_steps(ws, stream, args.steps, head["velocity_iterations"]))
        ws.close()
        sleep_on = {"value": total_bodies * args.steps / (ms_s / 1e3), "unit": UNIT, "ms_per_step": ms_s / args.steps,
                    "solver": head["solver"], "velocity_iterations": head["velocity_iterations"],
                    "note": "same worlds and timed steps with sleeping allowed (b2World::SetAllowSleeping(true)); "
                            "sleeping bodies count as body-steps, as in the CPU sleep-on figure"}

    if rank == 0:
        peak, peak_kind = measured_peaks()
        step_bytes = float(np.mean(stage_bytes))
        kernel_ms = float(stage_ms[1])
        achieved = step_bytes / (kernel_ms / 1e3) / 1e9
        total_stage = float(stage_ms.sum())
        ratio = TRAFFIC_PER_ALGORITHMIC_BYTE[head["solver"]]
        roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": step_bytes * ratio, "peak_source": peak_kind,
                "traffic_note": f"DRAM bytes per launch stage, scaled from an ncu capture of StepKernel ({head['solver']} "
                                "solver) on the 1024-world case (traffic per algorithmic byte)",
                "kernel": "b2g::StepKernel",
                "algorithmic_bytes_per_launch": step_bytes,
                "launch_ms": kernel_ms,
                "note": "StepKernel's stage (every class of the plan) carries the step's persistent-state "
                        "traffic (collide commit, island solve, fixture sync, pair finding); its bytes per "
                        f"step over its CUDA-event duration, averaged over {STAGE_STEPS} steps after the timed "
                        "region",
                "stages": {k: {"ms": float(m), "share": float(m) / total_stage}
                           for k, m in zip(STAGE_KERNELS, stage_ms)}}
        line = {
            "metric": METRIC, "value": head["value"], "unit": UNIT, "n_gpus": world_size, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": head["ms_per_step"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": config_dict(args, worlds),
            "headline": {"solver": head["solver"], "warm_start": head["warm_start"],
                         "velocity_iterations": head["velocity_iterations"],
                         "residual_median": head["residual_median"],
                         "rule": "the fastest arm whose median velocity residual is no larger than the reference-"
                                 "order solver's at 8 iterations (that solver is bit-exact with the reference)"},
            "arms": {k: r for k, (r, _) in arms.items()},
            "coloured_search": searched,
            "learned_search": learned_search,
            "learned_training": learned_info,
            "residual_definition": "max over contact points of the natural-map residual in m/s: |vn - bias| on "
                                   "active normal points, |vt| on friction inside its cone, 0 at a solution; after "
                                   "the velocity iterations; median over worlds at the step after the timed window "
                                   "(the timed steps do not measure it)",
            "sleep_on": sleep_on,
            "roofline": roof,
            "e2e": head["e2e"],
            "gpu_launches": args.steps * launches_per_step(len(head["launch_plan"])),
            "clocks": clk.summary(),
        }
        if not args.no_cpu_baseline and world_size == 1:
            threads = os.cpu_count() or 1
            line["cpu_baseline"] = cpu_baseline(worlds, args.steps, args.warmup, threads)
            if sleep_on is not None:
                cs = cpu_baseline(workload(args, rank, allow_sleep=True), args.steps, args.warmup, threads, sleep=True)
                sleep_on["cpu"] = {"value": cs["value"], "ms_per_step": cs["ms_per_step"], "cores": cs["cores"],
                                   "kind": cs["kind"]}
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
