"""Benchmark: body-steps/s of the batched world step on one GB300.

Workload: 4,096 independent worlds (body counts log-uniform in [16, 512],
60/40 discs/rectangles, each with its own ground box and gravity U[5,15]),
dt = 1/60, 8 solver iterations, one sub-step.  The scene is first advanced
300 steps (untimed) so that the timed steps see settled piles with their
full contact load, not bodies in free fall.  One "step" = one
Solver.process-equivalent pass over all 4,096 worlds.

Under torchrun with N ranks (one GPU each), every rank builds the same
N x 4,096 worlds, keeps the share dealt to it by body count
(resolve2d_gb300/shard.py) and steps it with nothing exchanged (weak
scaling); value is all ranks' bodies over the slowest rank's time.

value      body-steps/s with the state resident in HBM, CUDA events around
           each step on the library's stream, L2 flushed (256 MiB write)
           between steps outside the timed events.
e2e        the same metric through the C ABI with pinned host buffers: every
           step takes its inputs (force and torque rows) from the host and
           returns its result (pose and momenta rows) to the host, in one
           r2d_batch_process_io call whose kernels read and write the pinned
           rows over the CPU-GPU link; the same frame as three calls
           (write rows, step, read rows) and the full-state round trip are
           reported beside it.
roofline   algorithmic HBM bytes of the world-step kernel per step
           (117 B per body-step: 77 B read, 40 B written) over its measured
           time, against the measured copy bandwidth.  The unit is one step's
           world-step launches (one per size class, run concurrently on their
           own streams), timed by the events around the step.
pos_error_vs_fp64  stated from the committed precision study
           (tests/precision_study.py: the long-horizon workload against the
           FP64 oracle, position error in body radii).
cpu_baseline  the CPU oracle (the C++ restatement of the reference's step,
           in the reference's own constraint order) on this host's cores,
           from the same settled state, for about ten seconds.

--impl reference times that CPU step alone (the reference is Zig and cannot
be built here) and prints its own line.

--workload config1 | config2 measures one large world instead (the
12,001-body pyramid with falling discs; the 200,004-body box with chains and
motors), which the library steps on its grid pipeline: same metric, same
keys, CUDA events around each step (the pipeline's host round trips are
inside them), no plain-path comparison (the workload is one world).
"""

from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)
# The library runs the size classes of a step on up to 16 streams at once;
# CUDA's default of 8 hardware work queues would serialise some of them.  It
# only takes effect before CUDA starts in this process.
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

SETTLE_STEPS = 300
BYTES_READ = 77   # pos 8, angle 4, momentum 8, ang. momentum 4, force+torque 12, AABB 16, mass/inertia/mu/dims 20, kind 1, id 4
BYTES_WRITE = 40  # pos 8, angle 4, momentum 8, ang. momentum 4, AABB 16
# The compulsory-traffic model of the hot-path scope (pose, momenta, mass,
# inertia, mu, shape and type read; pose and momenta written), without the
# stored AABB and the force rows this layout keeps in HBM.
BYTES_MODEL_72 = 72
METRIC = "body-steps/sec on 1 GB300, batched FP32 vs plain, at stated pos error vs FP64"
HEADLINE = "config3: 4096 worlds, counts log-uniform [16,512], dt 1/60, 8 iterations, settled 300 steps"
# single large worlds: (scene name, description, settle steps)
LARGE = {
    "config1": ("config1: one world, 10,000-box pyramid + 2,000 discs falling onto it (12,001 bodies), dt 1/60, "
                "10 iterations, settled 300 steps", 300),
    "config2": ("config2: one world, 200,004 bodies in a walled 2000x500 box, 5,000 chains of 20 distance joints "
                "+ 2,000 motors, dt 1/120, 8 iterations, settled 30 steps", 30),
}


def max_over_ranks(x: float, device: str = "cuda") -> float:
    """The largest of every rank's `x` (the timed region of the slowest rank);
    `x` itself with one process."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(x: float, device: str = "cuda") -> float:
    """The sum of every rank's `x`; `x` itself with one process."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def rank_scene(rank: int, world: int, per_rank: int = 4096):
    """The worlds one rank steps.  One process: the headline batch (seed 3,
    4,096 worlds).  N processes: the N x 4,096 worlds of the same generator and
    seed, dealt out by body count (weak scaling, nothing exchanged while
    stepping).  Every rank builds the same global batch and keeps its share."""
    from resolve2d_gb300 import scenes
    from resolve2d_gb300.shard import balanced_shards

    if world == 1:
        return scenes.config3(nworlds=per_rank)
    full = scenes.config3(nworlds=per_rank * world)
    return full.select(balanced_shards(np.diff(full.body_off), world)[rank])


def headline_config(bodies: int, worlds: int, ranks: int, rank0_bodies: int) -> dict:
    """The workload both arms print (the driver compares them key for key)."""
    return {"workload": HEADLINE, "bodies": int(bodies), "worlds": int(worlds),
            "settle": f"{SETTLE_STEPS} steps in the GPU's colour-major constraint order before timing; the CPU "
                      "arm settles on the oracle, bit-identical to the GPU's settled state",
            "l2": "GPU arm: flushed between timed steps (256 MiB write outside the events)",
            "parallelism": (f"worlds dealt to {ranks} GPUs by body count, {rank0_bodies} bodies on rank 0"
                            if ranks > 1 else "one GPU")}


def spawn_command(n: int, argv: list[str], port: int) -> list[str]:
    """This script under torch.distributed.run with n local ranks (one GPU
    each), as `bench.py --gpus n` starts itself when no launcher set
    WORLD_SIZE."""
    return [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", f"--nproc-per-node={n}",
            "--master-addr", "127.0.0.1", f"--master-port={port}", os.path.abspath(__file__), *argv]


def free_port() -> int:
    import socket

    with socket.socket() as so:
        so.bind(("127.0.0.1", 0))
        return so.getsockname()[1]


def dry_run(args):
    """--dry-run: the rank logic alone, on the host (gloo): every rank builds
    its share of the global batch and the ranks reduce their body counts and
    a stand-in time as the timed run does; rank 0 prints the totals.  No
    GPU is touched; it checks a multi-rank launch before spending GPUs."""
    rank, world, _ = dist_env()
    import torch.distributed as dist

    if world > 1:
        dist.init_process_group("gloo")
    try:
        sc = rank_scene(rank, world, per_rank=args.dry_run_worlds)
        t = max_over_ranks(1.0 + 0.5 * rank, device="cpu")
        nb_all = int(round(sum_over_ranks(sc.nbodies, device="cpu")))
        nw_all = int(round(sum_over_ranks(sc.nworlds, device="cpu")))
        if rank == 0:
            print(json.dumps({"dry_run": True, "n_gpus": world, "worlds": nw_all, "bodies": nb_all,
                              "rank0_bodies": sc.nbodies, "slowest_rank_time": t}), flush=True)
    finally:
        if world > 1:
            dist.destroy_process_group()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines: list[str] = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                smax.append(float(p[2]))
            except ValueError:
                continue
            for nm, v in zip(names, p[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    p = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def traffic_from_profile():
    p = os.path.join(REPO, "profiles", "world_step_traffic.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return d.get("bytes_per_body_step")
    return None


def cpu_threads() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


def _with_constraints(sc) -> bool:
    """The oracle's batch runner steps bodies only; a scene with joints or
    exclusions (one world) steps through a whole oracle solver instead."""
    return bool(sc.jtype.size or sc.xpairs.size)


def _solver_run(sc, state, steps, order=None):
    """(seconds, final state) of `steps` oracle steps of a one-world scene with
    its joints and exclusions, on one thread, in the reference's order (or
    `order`)."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle as O

    if sc.nworlds != 1:  # Oracle.from_scene takes world 0 only
        raise ValueError(f"a scene with joints or exclusions is timed as one world, not {sc.nworlds}")
    o = O.Oracle.from_scene(sc)
    if state is not None:
        o.set_state(np.ascontiguousarray(state, np.float32))
    t0 = time.perf_counter()
    for _ in range(steps):
        st = o.process(sc.dt, sc.sub_steps, sc.iters, O.ORDER_REFERENCE if order is None else order)
        if st:
            raise RuntimeError(f"the oracle returned status {st}")
    return time.perf_counter() - t0, o.state()


def settle_scene(sc, steps):
    """Advance the scene `steps` steps on the CPU oracle (all host threads) in
    the GPU's colour-major constraint order, which the GPU reproduces bit for
    bit: both arms then time the same settled state."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle as O

    if _with_constraints(sc):
        return _solver_run(sc, None, steps, order=O.ORDER_COLOUR)[1]
    _, state, st = O.batch_run(sc, steps, cpu_threads(), order=O.ORDER_COLOUR)
    if st:
        raise RuntimeError(f"the oracle returned status {st}")
    return state.reshape(13, sc.nbodies)


def oracle_time(sc, state, steps, threads):
    """Seconds the oracle takes for `steps` steps of every world from `state`,
    in the reference's own constraint order (joints, then manifolds, in
    insertion and discovery order, lib.zig:226-236): the reference's step,
    without the colouring that the colour-major order adds."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle as O

    if _with_constraints(sc):
        return _solver_run(sc, state, steps)[0]
    secs, _, st = O.batch_run(sc, steps, threads, state_in=state, order=O.ORDER_REFERENCE)
    if st:
        raise RuntimeError(f"the oracle returned status {st}")
    return secs


def one_core_baseline(sc, state) -> dict:
    """The oracle's step on one thread (the reference itself is single-threaded),
    on a bounded sample: the first worlds holding about a tenth of the bodies,
    for about five seconds."""
    sub_w = int(np.searchsorted(sc.body_off, sc.nbodies // 10)) + 1
    sub = sc.worlds(0, min(sub_w, sc.nworlds))
    sub_state = np.ascontiguousarray(state[:, : sub.nbodies])
    one = oracle_time(sub, sub_state, 1, 1)
    steps = max(1, min(50, int(5.0 / max(one, 1e-3))))
    secs = oracle_time(sub, sub_state, steps, 1)
    return {"value": sub.nbodies * steps / secs, "unit": "body-steps/s", "seconds": secs,
            "sample": f"worlds 0..{sub.nworlds - 1} ({sub.nbodies} bodies) x {steps} steps on one thread"}


def stated_pos_error():
    """The f32-vs-FP64 position error the metric is stated at, from the
    committed precision study (tests/precision_study.py on the 16,384-world
    long-horizon workload)."""
    p = os.path.join(REPO, "profiles", "precision_config4.json")
    if not os.path.exists(p):
        return None
    with open(p) as f:
        d = json.load(f)
    out = {"source": "profiles/precision_config4.json (tests/precision_study.py)", "unit": "body radii",
           "oracle_worlds": d.get("oracle_worlds")}
    for step, modes in d.get("checkpoints", {}).items():
        out[f"step_{step}"] = {m: v["pos_error_vs_fp64_radii"] for m, v in modes.items()}
    return out


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from resolve2d_gb300 import build as B
    from resolve2d_gb300 import scenes

    B.build_oracle()
    if args.workload in LARGE:
        sc = getattr(scenes, args.workload)()
        workload, settle = LARGE[args.workload]
        config = {"workload": workload, "bodies": sc.nbodies, "worlds": sc.nworlds}
    else:
        # the GPU arm's workload: N x 4,096 worlds under N ranks; the CPU arm
        # times the first 4,096 of them (the same generator and seed), a
        # bounded sample with the same per-world distribution
        sc = scenes.config3(seed=3)
        settle = SETTLE_STEPS
        full_bodies = sc.nbodies if world == 1 else scenes.config3(nworlds=4096 * world).nbodies
        rank0 = rank_scene(0, world).nbodies if world > 1 else sc.nbodies
        config = headline_config(full_bodies, 4096 * world, world, rank0)
    threads = cpu_threads()
    state = settle_scene(sc, settle)
    # each step: one full pass over all 4,096 worlds
    for _ in range(args.warmup):
        oracle_time(sc, state, 1, threads)
    secs = oracle_time(sc, state, args.steps, threads)
    bsteps = sc.nbodies * args.steps
    v = bsteps / secs
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "body-steps/s", "n_gpus": 0,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * secs / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded)",
        "config": config,
        "cpu_baseline": {"value": v, "unit": "body-steps/s", "cores": 1 if _with_constraints(sc) else threads,
                         "kind": "port",
                         "sample": f"{sc.nworlds} worlds ({sc.nbodies} bodies) x {args.steps} steps from the settled "
                                   "state; C++ restatement of Solver.process in the reference's own constraint "
                                   "order (Zig toolchain absent)"},
        "e2e": {"value": v, "unit": "body-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    if sc.nworlds > 1:
        line["cpu_baseline"]["one_core"] = one_core_baseline(sc, state)
    print(json.dumps(line), flush=True)


def run_large(args):
    """One large world on the grid pipeline (--workload config1 / config2)."""
    rank, world, local = dist_env()
    import torch

    torch.cuda.set_device(local)
    from resolve2d_gb300 import build as B
    from resolve2d_gb300 import scenes
    from resolve2d_gb300.engine import World

    B.build_library()
    sc = getattr(scenes, args.workload)()
    workload, settle = LARGE[args.workload]
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    batch = World.from_scene(sc, stream=stream.cuda_stream)
    for _ in range(settle):
        batch.process(sc.dt, sc.sub_steps, sc.iters)
    batch.sync()
    settled = batch.read_state()
    nb = sc.nbodies
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    for _ in range(args.warmup):
        batch.process(sc.dt, sc.sub_steps, sc.iters)
    batch.sync()
    batch.write_state(settled)
    batch.sync()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    clocks = ClockSampler(local)
    torch.cuda.synchronize()
    clocks.start()
    torch.cuda.profiler.start()
    t0 = time.perf_counter()
    launches = 0
    for k in range(args.steps):
        flush.zero_()
        starts[k].record(stream)
        batch.process(sc.dt, sc.sub_steps, sc.iters)
        ends[k].record(stream)
        launches += batch.launches_per_step()
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    torch.cuda.profiler.stop()
    batch.sync()
    clk = clocks.stop()
    dev_s = sum(s_.elapsed_time(e_) for s_, e_ in zip(starts, ends)) / 1e3
    step_s = dev_s / args.steps
    value = nb * args.steps / dev_s

    e2e_steps = max(3, min(args.steps, 10))
    forces_in = torch.zeros((3, nb), dtype=torch.float32).pin_memory().numpy()
    pose_out = torch.empty((6, nb), dtype=torch.float32).pin_memory().numpy()
    batch.write_state(settled)
    batch.sync()
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    for _ in range(e2e_steps):
        batch.process_io(sc.dt, sc.sub_steps, sc.iters, forces_in, pose_out)
    batch.sync()
    e2e_v = nb * e2e_steps / (time.perf_counter() - t1)

    peak, peak_src = measured_peaks()
    achieved = (BYTES_READ + BYTES_WRITE) * nb / step_s / 1e9
    line = {
        "metric": METRIC, "value": value, "unit": "body-steps/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * step_s, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
        "config": {"workload": workload, "bodies": nb, "worlds": sc.nworlds, "joints": int(len(sc.jtype)),
                   "l2": "flushed between timed steps (256 MiB write outside the events)",
                   "path": "grid pipeline (one world larger than a CTA's shared memory)"},
        "gpu_launches": launches,
        "wall_s_timed_loop": wall,
        "e2e": {"value": e2e_v, "unit": "body-steps/s", "h2d_bytes_per_step": 12 * nb, "d2h_bytes_per_step": 24 * nb,
                "inputs": "force and torque rows (pinned)", "results": "pose and momenta rows (pinned)",
                "call": "r2d_solver_process_io (grid-pipeline worlds copy the rows around the step)"},
        "plain_one_world_per_launch": None,
        "roofline": {"bound": "hbm", "kernel": "grid pipeline (all launches of one step)",
                     "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_source": peak_src, "traffic": None, "bytes_per_body_step": BYTES_READ + BYTES_WRITE},
        "clocks": clk,
    }
    if not args.no_cpu_baseline:
        threads = cpu_threads()
        one = oracle_time(sc, settled, 1, threads)
        cpu_steps = max(2, min(200, int(10.0 / max(one, 1e-3))))
        secs = oracle_time(sc, settled, cpu_steps, threads)
        line["cpu_baseline"] = {"value": nb * cpu_steps / secs, "unit": "body-steps/s", "cores": 1,
                                "kind": "port", "seconds": secs,
                                "sample": f"the world x {cpu_steps} steps from the settled state on one core (the "
                                          "oracle threads over worlds; C++ restatement of Solver.process in the "
                                          "reference's own constraint order)"}
    print(json.dumps(line), flush=True)


def plain_drop_in(name: str, stream, no_cpu: bool) -> dict:
    """One large world (config 1 or 2) through the single-world entry points
    (r2d_solver_*), the drop-in for Solver.process, which steps it on the
    grid pipeline: settled as in --workload, then 10 steps timed by CUDA
    events on the library's stream (the pipeline's host round trips inside
    them), L2 flushed between steps.  Beside it, one step of the CPU oracle
    from the same settled state on one core, in the reference's order."""
    import torch
    from resolve2d_gb300 import scenes
    from resolve2d_gb300.engine import World

    sc = getattr(scenes, name)()
    desc, settle = LARGE[name]
    w = World.from_scene(sc, stream=stream.cuda_stream)
    for _ in range(settle):
        w.process(sc.dt, sc.sub_steps, sc.iters)
    w.sync()
    settled = w.read_state()
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    steps = 10
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    torch.cuda.synchronize()
    for a, b in ev:
        flush.zero_()
        a.record(stream)
        w.process(sc.dt, sc.sub_steps, sc.iters)
        b.record(stream)
    w.sync()
    torch.cuda.synchronize()
    secs = sum(a.elapsed_time(b) for a, b in ev) / 1e3
    out = {"workload": desc, "bodies": sc.nbodies, "joints": int(sc.jtype.size), "steps": steps,
           "ms_per_step": 1e3 * secs / steps, "value": sc.nbodies * steps / secs, "unit": "body-steps/s",
           "call": "r2d_solver_process (grid pipeline)", "launches_per_step": w.launches_per_step()}
    w.close()
    if not no_cpu:
        cpu = oracle_time(sc, settled, 1, 1)
        out["cpu_one_core"] = {"value": sc.nbodies / cpu, "unit": "body-steps/s", "seconds": cpu,
                               "sample": "one step from the settled state on one core, reference order"}
    return out


def arg_parser() -> argparse.ArgumentParser:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-autotune", action="store_true", help="keep the default threads per size class")
    ap.add_argument("--no-precision", action="store_true", help="accepted for older command lines; no effect")
    ap.add_argument("--plain-worlds", type=int, default=64,
                    help="worlds stepped one per launch for the plain-path comparison")
    ap.add_argument("--workload", default="config3", choices=["config3", *LARGE],
                    help="config3 (the headline batch) or one large world on the grid pipeline")
    ap.add_argument("--no-plain-drop-in", action="store_true",
                    help="skip the config 1 / config 2 single-world lines inside the headline line")
    ap.add_argument("--dry-run", action="store_true",
                    help="the multi-rank logic alone on the host (gloo), no GPU: prints the ranks' totals")
    ap.add_argument("--dry-run-worlds", type=int, default=64, help="worlds per rank in --dry-run")
    return ap


def main():
    args = arg_parser().parse_args()
    rank, world, _ = dist_env()
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        # one process per GPU: start this script under torch.distributed.run
        sys.exit(subprocess.call(spawn_command(args.gpus, sys.argv[1:], free_port())))
    if "WORLD_SIZE" in os.environ and world != args.gpus:
        raise SystemExit(f"--gpus {args.gpus} but the launcher started {world} ranks")
    if args.dry_run:
        return dry_run(args)
    if args.impl == "reference":
        return run_reference(args)
    if args.workload in LARGE:
        return run_large(args)

    rank, world, local = dist_env()
    import torch

    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    from resolve2d_gb300 import build as B
    from resolve2d_gb300 import scenes
    from resolve2d_gb300.engine import Batch, World

    B.build_library()
    sc = rank_scene(rank, world)
    # a dedicated stream: the library launches on it and the CUDA events below
    # are recorded on it (the legacy default stream has handle 0, which the
    # library would replace with a stream of its own)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    batch = Batch.from_scene(sc, stream=stream.cuda_stream)
    # settle (untimed): bring the worlds to their loaded state
    for _ in range(SETTLE_STEPS):
        batch.process(sc.dt, sc.sub_steps, sc.iters)
    batch.sync()
    settled = batch.read_state()
    # pick each size class's threads per CTA on the settled worlds (untimed;
    # the state is restored)
    if not args.no_autotune:
        batch.autotune(sc.dt, sc.sub_steps, sc.iters, trial_steps=8)
    nb = sc.nbodies

    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    for _ in range(args.warmup):
        batch.process(sc.dt, sc.sub_steps, sc.iters)
    batch.sync()
    batch.write_state(settled)
    batch.sync()

    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    clocks = ClockSampler(local)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clocks.start()
    # cudaProfilerStart/Stop bracket the timed steps: a profiler started with
    # its capture off (ncu --profile-from-start off) sees only these launches
    torch.cuda.profiler.start()
    t0 = time.perf_counter()
    for k in range(args.steps):
        flush.zero_()
        starts[k].record(stream)
        batch.process(sc.dt, sc.sub_steps, sc.iters)
        ends[k].record(stream)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    torch.cuda.profiler.stop()
    batch.sync()
    ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    dev_s = sum(ms) / 1e3
    dev_s = max_over_ranks(dev_s)
    clk = clocks.stop()
    nb_all = int(round(sum_over_ranks(nb)))  # bodies stepped by all ranks together
    nw_all = int(round(sum_over_ranks(sc.nworlds)))
    value = nb_all * args.steps / dev_s
    launches = batch.launches_per_step() * args.steps

    # End to end through the C ABI with pinned host buffers.  Each step
    # writes its inputs, the force and torque rows (12 B/body), and reads its
    # result, the pose and momenta rows (24 B/body), as a frame loop does with
    # r2d_batch_write_state_fields / process / read_state_fields; the whole
    # state both ways (52 B/body each) is timed beside it.
    e2e_steps = max(3, min(args.steps, 10))

    def timed_e2e(step_fn):
        batch.write_state(settled)
        batch.sync()
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        for _ in range(e2e_steps):
            step_fn()
        batch.sync()
        return nb_all * e2e_steps / max_over_ranks(time.perf_counter() - t1)

    forces_in = torch.zeros((3, nb), dtype=torch.float32).pin_memory().numpy()
    pose_out = torch.empty((6, nb), dtype=torch.float32).pin_memory().numpy()
    state_io = torch.empty((13, nb), dtype=torch.float32).pin_memory().numpy()
    state_io[...] = settled

    def frame_step():  # one call: the step reads the pinned force rows and writes the result rows itself
        batch.process_io(sc.dt, sc.sub_steps, sc.iters, forces_in, pose_out)

    def fields_step():
        batch.write_fields(6, forces_in)
        batch.process(sc.dt, sc.sub_steps, sc.iters)
        batch.read_fields(0, 6, pose_out)

    def full_step():
        batch.write_state(state_io)
        batch.process(sc.dt, sc.sub_steps, sc.iters)
        batch.read_state(state_io)

    e2e_v = timed_e2e(frame_step)
    e2e_three = timed_e2e(fields_step)
    e2e_full = timed_e2e(full_step)

    # plain path: the same worlds, one world per launch
    plain = None
    if args.plain_worlds > 0:
        pw = min(args.plain_worlds, sc.nworlds)
        worlds = [World.from_scene(sc.world(w), stream=stream.cuda_stream) for w in range(pw)]
        for i, w in enumerate(worlds):  # first process plans the launch (untimed)
            w.process(sc.dt, sc.sub_steps, sc.iters)
            w.sync()
            b0, b1 = sc.body_off[i], sc.body_off[i + 1]
            w.write_state(np.ascontiguousarray(settled[:, b0:b1]))
        torch.cuda.synchronize()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        for w in worlds:
            w.process(sc.dt, sc.sub_steps, sc.iters)
        ev1.record(stream)
        torch.cuda.synchronize()
        nbp = int(sc.body_off[pw])
        plain = nbp / (ev0.elapsed_time(ev1) / 1e3)
        for w in worlds:
            w.close()

    peak, peak_src = measured_peaks()
    step_s = dev_s / args.steps
    achieved = (BYTES_READ + BYTES_WRITE) * nb / step_s / 1e9
    traffic = traffic_from_profile()
    line = {
        "metric": METRIC, "value": value, "unit": "body-steps/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * step_s, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
        "config": headline_config(nb_all, nw_all, world, nb),
        "tuning": {"tiles": "threads per CTA of each size class autotuned on the settled worlds"
                   if not args.no_autotune else "default threads per size class",
                   "cuda_device_max_connections": os.environ.get("CUDA_DEVICE_MAX_CONNECTIONS")},
        "gpu_launches": launches,
        "wall_s_timed_loop": wall,
        "e2e": {"value": e2e_v, "unit": "body-steps/s", "h2d_bytes_per_step": 12 * nb_all,
                "d2h_bytes_per_step": 24 * nb_all,
                "inputs": "force and torque rows (pinned)", "results": "pose and momenta rows (pinned)",
                "call": "r2d_batch_process_io (the step reads and writes the pinned rows over the CPU-GPU link)",
                "three_calls": {"value": e2e_three, "call": "write_state_fields, process, read_state_fields"},
                "full_state": {"value": e2e_full, "h2d_bytes_per_step": 52 * nb_all,
                               "d2h_bytes_per_step": 52 * nb_all}},
        "plain_one_world_per_launch": {"value": plain, "unit": "body-steps/s", "worlds": args.plain_worlds,
                                       "batched_over_plain": (value * nb / nb_all) / plain if plain else None},
        "roofline": {"bound": "hbm", "kernel": "world_step_kernel (the size-class launches of one step)",
                     "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_source": peak_src,
                     "traffic": None if traffic is None else traffic * nb,
                     "bytes_per_body_step": BYTES_READ + BYTES_WRITE,
                     "model_72": {"bytes_per_body_step": BYTES_MODEL_72,
                                  "achieved": BYTES_MODEL_72 * nb / step_s / 1e9,
                                  "frac": BYTES_MODEL_72 * nb / step_s / 1e9 / peak}},
        "clocks": clk,
    }
    line["pos_error_vs_fp64"] = stated_pos_error()
    if rank == 0 and world == 1 and not args.no_plain_drop_in:
        line["plain_drop_in"] = {w: plain_drop_in(w, stream, args.no_cpu_baseline) for w in LARGE}
    if rank == 0 and not args.no_cpu_baseline:
        threads = cpu_threads()
        one = oracle_time(sc, settled, 1, threads)
        cpu_steps = max(2, min(200, int(10.0 / max(one, 1e-3))))
        secs = oracle_time(sc, settled, cpu_steps, threads)
        line["cpu_baseline"] = {"value": nb * cpu_steps / secs, "unit": "body-steps/s", "cores": threads,
                                "kind": "port", "seconds": secs,
                                "sample": f"all {sc.nworlds} worlds x {cpu_steps} steps from the settled state "
                                          "(C++ restatement of Solver.process in the reference's own constraint order; "
                                          "Zig toolchain absent)"}
        line["cpu_baseline"]["one_core"] = one_core_baseline(sc, settled)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
