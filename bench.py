"""Benchmark of the GB300 Box2D step: body-steps/s on one GB300.

Workload (default): many pyramids with rain -- a 20x20 grid of 10-row pyramids of 0.5 m
boxes (22000 dynamic bodies) plus 2000 falling circles, dt 1/60 s, 4 substeps, float32.
One timed "step" is one b2World_Step of that world. Inputs (the world) are resident on the
device when the timed region starts; each timed step is bracketed by CUDA events on the
library's stream, and L2 is flushed (a 256 MiB write) between timed steps, outside them.

`value` = dynamic bodies x timed steps / summed device-timed step time, all ranks.
`e2e`   = the same metric with, per step, b2World_Step followed by the body move-event read
          (every awake body transform copied to host), wall-clocked; the byte counts are the
          library's own host<->device traffic plus the move events.
`roofline` is for the solver (constraint preparation through impulse storage), the
dominant device stage: algorithmic bytes from the reference data layout
(S*(120 Nb + 708 Nc + 604 Nj) + 364 Nc per step; +260 Nc with restitution) over its
CUDA-event time, against the measured HBM copy bandwidth.
`cpu_baseline` times the reference itself -- its own sources compiled on this machine
(oracle/_ref/libref.so, Release flags, the SIMD its core.h picks) with its built-in
scheduler on one worker per host core -- on a bounded sample of the same workload, and
`cpu_port` the CPU oracle (the C restatement) beside it. Where the reference build is
missing the oracle stands in and `cpu_baseline.kind` says "port".
`pose_error` compares the GPU world with the reference world after the same number of
steps (the end of the timed window): largest position and rotation difference.

--impl reference runs that CPU step alone with the same line format.
Multi-GPU: independent replicas per rank (the step of one world does not shard).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

import box2d_gb300 as B  # noqa: E402

# untimed steps before the warm-up: the many-pyramids rain reaches the pyramids after about
# 150 steps, so the timed window starts where the scene's contact churn does
START_STEPS = {"many_pyramids": 200, "large_pyramid": 0, "joint_grid": 0, "batch_worlds": 0, "diff_batch": 0}

WORKLOADS = {
    # name: (kind, a, b, c, seed, flags, description)
    "many_pyramids": (B.MANY_PYRAMIDS_RAIN, 20, 10, 2000, 0, 0,
                      "20x20 grid of 10-row pyramids of 0.5 m boxes + 2000 rain circles"),
    "large_pyramid": (B.LARGE_PYRAMID, 100, 1, 0, 0, 0, "100-row pyramid of 5050 boxes on a 200 m segment"),
    "joint_grid": (B.JOINT_GRID_MIXED, 100, 3000, 0, 0, 0,
                   "100x100 revolute circle grid + 3000 mixed shapes"),
    "batch_worlds": (B.BATCH_WORLD, 0, 0, 0, 12345, 0,
                     "independent worlds of 10-400 boxes, circles and capsules in a 3-segment container"),
    "diff_batch": (B.RAMP_WORLD, 8, 8, 0, 12345, 0,
                   "differentiable batch: worlds of 8 x 8 boxes on a 10-30 degree ramp, forward + adjoint "
                   "(gradient of |final center of mass - target|^2 w.r.t. initial velocities and frictions)"),
}


# DRAM bytes (read + write) per step of the solver-stage kernels (component analysis, bins,
# cluster assignment, cluster solve) in the timed window, from one ncu capture of each
# workload's timed steps (profiles/solver_traffic_timed_steps.md: command and per-kernel split)
SOLVER_TRAFFIC = {"many_pyramids": 43.45e6, "large_pyramid": 3.48e6, "joint_grid": 18.56e6}


def peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return {"hbm_gbs": float(d["hbm_gbs"]), "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons while running."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.summary = {"sm_mhz": None, "sm_max_mhz": None, "reasons": []}
        if self.proc is None:
            return
        time.sleep(0.25)
        self.proc.terminate()
        out, _ = self.proc.communicate(timeout=5)
        rows = [r.split(",") for r in out.strip().splitlines() if r.strip()]
        sm = [float(r[1]) for r in rows if len(r) > 2 and r[1].strip().replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if len(r) > 2 and r[2].strip().replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for k, name in enumerate(names):
                if len(r) > 5 + k and "Active" in r[5 + k] and "Not" not in r[5 + k]:
                    reasons.add(name)
        self.summary = {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                        "reasons": sorted(reasons), "samples": len(rows)}


def algorithmic_bytes(counters: np.ndarray, awake: int, substeps: int, restitution: bool) -> float:
    """Per-step compulsory bytes of the solver stage (solver data of the reference)."""
    colors = counters[4:28]
    joints = int(counters[3])
    nc = int(colors.sum()) - joints
    b = substeps * (120 * awake + 708 * nc + 604 * joints) + 364 * nc
    if restitution:
        b += 260 * nc
    return float(b)


HOST_PHASES = ["tree_upload", "pair_query", "contact_create", "tree_rebuild", "narrowphase", "state_pass", "uploads",
               "solver", "enlarge"]


def run_gpu(args, rank: int, world_size: int) -> dict:
    import torch

    dev = rank % max(1, torch.cuda.device_count())
    torch.cuda.set_device(dev)
    kind, a, b, c, seed, flags, desc = WORKLOADS[args.workload]
    lib = B.load_library()
    scene = B.Scene(lib, kind, a, b, c, seed, flags)
    dyn = scene.dynamic_count
    stream = torch.cuda.ExternalStream(lib.b2p_stream(scene.world_id))
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")
    scene.step(args.start_step)
    for _ in range(args.warmup):
        scene.step()
    torch.cuda.synchronize()
    scene.timings(reset=True)
    scene.host_profile(reset=True)
    counters_before = scene.counters()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    solver_ms = 0.0
    alg_bytes = 0.0
    if world_size > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    if args.profile_timed:
        torch.cuda.profiler.start()  # ncu --profile-from-start off captures the timed steps only
    with ClockSampler(dev) as clocks:
        for k in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            starts[k].record(stream)
            scene.step()
            ends[k].record(stream)
            alg_bytes += algorithmic_bytes(scene.counters(), dyn, 4, False)
        torch.cuda.synchronize()
    if args.profile_timed:
        torch.cuda.profiler.stop()
    if world_size > 1:
        torch.distributed.barrier()
    step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    stage_ms, traffic = scene.timings(reset=True)
    host_ms = scene.host_profile(reset=True)
    window_state = scene.state()  # at the end of the timed window, for the CPU comparison
    total_ms = float(sum(step_ms))
    solver_ms = float(stage_ms[2])
    launches = int(traffic[2])

    # end to end: step + the step's body move events (b2World_GetBodyEvents, every awake
    # body's transform) read back through the public API, wall clock
    scene.timings(reset=True)
    events = np.zeros((scene.body_count, 4), np.float32)
    t0 = time.perf_counter()
    e2e_steps = max(1, min(args.steps, 200))
    move_bytes = 0
    step_s = 0.0
    for _ in range(e2e_steps):
        t1 = time.perf_counter()
        scene.step()
        step_s += time.perf_counter() - t1
        ev = scene.move_events(events)
        move_bytes += ev.nbytes
    e2e_s = time.perf_counter() - t0
    _, e2e_traffic = scene.timings(reset=True)
    counters = scene.counters()
    scene.close()
    pk = peaks()
    achieved = alg_bytes / (solver_ms * 1e-3) / 1e9 if solver_ms > 0 else 0.0
    return {
        "total_ms": total_ms, "step_ms": step_ms, "dyn": dyn, "solver_ms": solver_ms, "alg_bytes": alg_bytes,
        "achieved_gbs": achieved, "peak": pk, "launches": launches, "clocks": clocks.summary,
        "e2e_value": dyn * e2e_steps / e2e_s, "e2e_h2d": float(e2e_traffic[0]) / e2e_steps,
        "e2e_d2h": float(e2e_traffic[1]) / e2e_steps, "counters": counters.tolist(),
        "stage_ms": stage_ms.tolist(), "desc": desc, "counters_before": counters_before.tolist(),
        "host_ms": host_ms.tolist(), "e2e_step_ms": 1e3 * step_s / e2e_steps,
        "e2e_read_ms": 1e3 * (e2e_s - step_s) / e2e_steps, "window_state": window_state,
    }


def run_batch(args) -> dict:
    """Batched worlds: `args.worlds` independent worlds (body count drawn from 10-400 per
    world, seed 12345 + index) stepped together with b2World_StepBatch on all host cores,
    and, for comparison, the same worlds stepped one after the other (the plain per-world
    loop). Wall clock: every world's step returns only after its device work is done."""
    import ctypes

    import torch

    torch.cuda.set_device(0)
    lib = B.load_library()
    n = args.worlds
    threads = args.threads if args.threads > 0 else 4 * max(1, os.cpu_count() or 1)
    dt = 1.0 / 60.0

    def make_worlds():
        return [B.Scene(lib, B.BATCH_WORLD, 0, 0, 0, 12345 + i, 0) for i in range(n)]

    # the plain per-world loop: b2World_Step on each world in turn, over the same window
    # (warm-up steps, then `steps` timed) as the batched run below, on worlds built anew
    scenes = make_worlds()
    handles = (ctypes.c_int * n)(*[s.handle for s in scenes])
    lib.b2s_step_batch(handles, n, dt, 4, args.warmup, threads)
    plain_steps = args.steps
    t0 = time.perf_counter()
    for s in scenes:
        s.step(plain_steps)
    plain_s = time.perf_counter() - t0
    for s in scenes:
        s.close()
    scenes = make_worlds()
    handles = (ctypes.c_int * n)(*[s.handle for s in scenes])
    dyn = sum(s.dynamic_count for s in scenes)
    lib.b2s_step_batch(handles, n, dt, 4, args.warmup, threads)
    for s in scenes:
        s.timings(reset=True)
        s.host_profile(reset=True)
    prof = np.zeros(17, np.float32)
    lib.b2p_batch_profile(prof.ctypes.data, 1)
    launches0 = float(prof[5])
    with ClockSampler(0) as clocks:
        t0 = time.perf_counter()
        lib.b2s_step_batch(handles, n, dt, 4, args.steps, threads)
        batch_s = time.perf_counter() - t0
    lib.b2p_batch_profile(prof.ctypes.data, 1)
    # state of the first worlds after warm-up + timed steps, for the CPU comparison
    states = {i: scenes[i].state() for i in range(min(n, 120))}
    h2d = d2h = 0
    for s in scenes:
        _, traffic = s.timings(reset=True)
        h2d += int(traffic[0])
        d2h += int(traffic[1])
    launches = int(prof[5] - launches0)
    # host time of the step's phases summed over the worlds (thread time, not wall time)
    host_cpu = np.zeros(10, np.float64)
    for s in scenes:
        host_cpu += s.host_profile(reset=True)
    host_cpu_ms = {k: float(v) / args.steps for k, v in zip(
        ["tree_upload", "pair_query", "contact_create", "tree_rebuild", "narrowphase", "state_pass", "uploads",
         "solver", "enlarge"], host_cpu)}
    profile = {k: float(v) / args.steps for k, v in
               zip(["begin", "pairs", "collide", "finish", "flush", "_", "flush_assembly", "flush_wait", "_", "_", "_", "_",
                       "flush_plan", "flush_layout", "flush_stage", "flush_issue", "flush_deliver"], prof) if k != "_"}
    # end to end: the batched step plus every world's move events
    cap = sum(s.body_count for s in scenes)
    events = np.zeros((cap, 4), np.float32)
    e2e_steps = max(1, min(args.steps, 20))
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        lib.b2s_step_batch(handles, n, dt, 4, 1, threads)
        lib.b2s_move_events_many(handles, n, events.ctypes.data, cap)
    e2e_s = time.perf_counter() - t0
    for s in scenes:
        s.close()
    return {"dyn": dyn, "batch_s": batch_s, "plain_s": plain_s, "plain_steps": plain_steps, "threads": threads,
            "launches": launches, "h2d": h2d / args.steps, "d2h": d2h / args.steps, "clocks": clocks.summary,
            "e2e_value": dyn * e2e_steps / e2e_s, "profile": profile, "states": states, "host_cpu_ms": host_cpu_ms}


def run_diff(args) -> dict:
    """Differentiable batch: `args.worlds` ramp worlds (seed 12345 + index) stepped forward
    `args.steps` steps with the tape recording (b2World_StepBatch on all host cores), then
    the adjoint of every recorded step of every world (one launch per step). Wall clock of
    both halves through the public API, plus the adjoint kernels' device time."""
    import numpy as np

    import torch

    from box2d_gb300.diff import DiffBatch

    torch.cuda.set_device(0)
    lib = B.load_library()
    n = args.worlds
    threads = args.threads if args.threads > 0 else 4 * max(1, os.cpu_count() or 1)
    batch = DiffBatch(lib, B.RAMP_WORLD, 8, 8, 0, [12345 + i for i in range(n)])
    dyn = sum(s.dynamic_count for s in batch.scenes)
    masks = [np.arange(s.body_count) > 0 for s in batch.scenes]
    targets = []
    for s in batch.scenes:
        t = np.zeros(2, np.float32)
        lib.b2s_target(s.handle, t.ctypes.data)
        targets.append(t)
    v0, f0 = batch.velocities(), batch.friction()

    def forward(steps, record=True):
        batch.reset()
        batch.set_velocities(v0)
        batch.set_friction(f0)
        t0 = time.perf_counter()
        batch.step(steps, threads=threads, record=record)
        return time.perf_counter() - t0

    def backward():
        cs = batch.centers()
        grads = []
        for w, c in enumerate(cs):
            d = c[masks[w]].astype(np.float64).mean(0) - targets[w]
            g = np.zeros_like(c)
            g[masks[w]] = (2.0 * d / masks[w].sum()).astype(np.float32)
            grads.append(g)
        t0 = time.perf_counter()
        gv, _, gf = batch.backward(grads)
        return time.perf_counter() - t0, gv, gf

    warm_steps = max(1, min(args.steps, 10))
    for _ in range(args.warmup):
        forward(warm_steps)
        backward()
    plain_s = forward(args.steps, record=False)
    prof = np.zeros(17, np.float32)
    lib.b2p_batch_profile(prof.ctypes.data, 1)
    launches0 = float(prof[5])
    with ClockSampler(0) as clocks:
        fwd_s = forward(args.steps)
        lib.b2p_batch_profile(prof.ctypes.data, 1)
        bwd_s, gv, gf = backward()
    fwd_launches = int(prof[5] - launches0)
    profile = {k: float(v) / args.steps for k, v in
               zip(["begin", "pairs", "collide", "finish", "flush", "_", "flush_assembly", "flush_wait", "_", "_", "_", "_",
                       "flush_plan", "flush_layout", "flush_stage", "flush_issue", "flush_deliver"], prof) if k != "_"}
    adj_ms, launches = batch.backward_ms()
    tape_bytes = 0
    for w in range(min(n, 8)):
        tape_bytes += len(batch.download_tape(w))
    tape_bytes = tape_bytes * n / min(n, 8)
    finite = all(np.isfinite(g).all() for g in gv) and all(np.isfinite(g).all() for g in gf)
    batch.close()
    return {"dyn": dyn, "fwd_s": fwd_s, "bwd_s": bwd_s, "plain_s": plain_s, "adj_ms": adj_ms,
            "launches": launches + fwd_launches, "threads": threads, "clocks": clocks.summary, "tape_bytes": tape_bytes,
            "finite": finite, "profile": profile}


REF_LIB = ROOT / "oracle" / "_ref" / "libref.so"
ORACLE_LIB = ROOT / "oracle" / "liboracle.so"


def cpu_impl() -> str:
    """'reference' when the reference build exists on this machine, else 'port' (oracle)."""
    return "reference" if REF_LIB.exists() else "port"


def cpu_threads() -> int:
    # the reference caps its worker count at B2_MAX_WORKERS = 32 (constants.h:18)
    return max(1, min(os.cpu_count() or 1, 32))


def _cpu_lib(impl: str):
    import ctypes

    lib = B.load_library(REF_LIB if impl == "reference" else ORACLE_LIB)
    if impl == "port":
        lib.b2o_set_threads.argtypes = [ctypes.c_int]
    return lib


def pose_error(a: np.ndarray, b: np.ndarray) -> dict:
    """Largest position (m) and rotation (cos/sin component) difference between two
    b2s_get_state snapshots, and whether the snapshots are bit-identical."""
    dp = float(np.abs(a[:, 0:2].astype(np.float64) - b[:, 0:2]).max()) if a.size else 0.0
    dq = float(np.abs(a[:, 2:4].astype(np.float64) - b[:, 2:4]).max()) if a.size else 0.0
    return {"max_position_m": dp, "max_rotation": dq, "bit_exact": bool(a.tobytes() == b.tobytes())}


def run_cpu_batch(args, budget_s: float, max_steps: int, impl: str, gpu_states=None) -> dict:
    """A CPU library on a sample of the batched workload's worlds (the first `sample` seeds),
    every host core stepping whole worlds in parallel, one world per task (each world
    single-threaded), as a batch of independent worlds runs on a CPU. ctypes releases the
    interpreter lock during each call. `gpu_states` (world index -> b2s_get_state after
    warm-up + steps) are compared with the CPU worlds after the same number of steps."""
    from concurrent.futures import ThreadPoolExecutor

    kind, a, b, c, seed, flags, desc = WORKLOADS[args.workload]
    lib = _cpu_lib(impl)
    if impl == "port":
        lib.b2o_set_threads(1)
    threads = cpu_threads()
    sample = min(args.worlds, 16 * threads, 120)  # both CPU libraries hold at most 128 worlds
    scenes = [B.Scene(lib, kind, a, b, c, seed + i, flags) for i in range(sample)]
    dyn = sum(s.dynamic_count for s in scenes)
    err = None
    with ThreadPoolExecutor(threads) as ex:
        list(ex.map(lambda s: s.step(max(1, args.warmup)), scenes))
        t0 = time.perf_counter()
        n = 0
        paused = 0.0
        while n < max_steps and time.perf_counter() - t0 < budget_s:
            list(ex.map(lambda s: s.step(), scenes))
            n += 1
            if gpu_states is not None and n == args.steps:
                t1 = time.perf_counter()
                errs = [pose_error(gpu_states[i], scenes[i].state()) for i in range(sample) if i in gpu_states]
                if errs:
                    err = {"max_position_m": max(e["max_position_m"] for e in errs),
                           "max_rotation": max(e["max_rotation"] for e in errs),
                           "bit_exact": all(e["bit_exact"] for e in errs), "worlds": len(errs)}
                paused += time.perf_counter() - t1
        dt = time.perf_counter() - t0 - paused
    for s in scenes:
        s.close()
    return {"value": dyn * n / dt, "steps": n, "seconds": dt, "dyn": dyn, "threads": threads, "worlds": sample,
            "pose_error": err}


def run_cpu_sample(args, budget_s: float, max_steps: int, impl: str, gpu_state=None) -> dict:
    """A CPU library on the same workload, bounded by `max_steps` and `budget_s`:
    impl 'reference' -- the reference build with its built-in scheduler on one worker per
    host core (b2WorldDef.workerCount; physics_world.c:307-314); impl 'port' -- the oracle
    with its data-parallel loops on every host core. Timing starts after the same untimed
    steps as the GPU run's timed window; `gpu_state` (b2s_get_state at the window's end) is
    compared with the CPU world after the same step count, outside the timed region."""
    kind, a, b, c, seed, flags, desc = WORKLOADS[args.workload]
    lib = _cpu_lib(impl)
    threads = cpu_threads()
    if impl == "reference":
        lib.b2s_set_workers(threads)
    else:
        lib.b2o_set_threads(threads)
    scene = B.Scene(lib, kind, a, b, c, seed, flags)
    if impl == "reference":
        lib.b2s_set_workers(0)
    scene.step(args.start_step)
    for _ in range(args.warmup):
        scene.step()
    err = None
    t0 = time.perf_counter()
    n = 0
    paused = 0.0
    while n < max_steps and time.perf_counter() - t0 < budget_s:
        scene.step()
        n += 1
        if gpu_state is not None and n == args.steps:
            t1 = time.perf_counter()
            err = pose_error(gpu_state, scene.state())
            err["step"] = args.start_step + args.warmup + args.steps
            paused += time.perf_counter() - t1
    dt = time.perf_counter() - t0 - paused
    dyn = scene.dynamic_count
    scene.close()
    if impl == "port":
        lib.b2o_set_threads(1)
    return {"value": dyn * n / dt, "steps": n, "seconds": dt, "dyn": dyn, "threads": threads, "pose_error": err}


def cpu_description(impl: str, threads: int, batched: bool) -> str:
    if impl == "reference":
        who = ("the reference built from its sources (-O3, NEON/SSE2 as its core.h selects), "
               + ("one single-threaded world per task" if batched else "built-in scheduler, workerCount"))
    else:
        who = "C oracle (restatement of the reference step)" + (", one world per task" if batched else "")
    return f"{who} on {threads} threads"


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=300)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="many_pyramids", choices=sorted(WORKLOADS))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--profile-timed", action="store_true",
                    help="bracket the timed steps with cudaProfilerStart/Stop (for ncu --profile-from-start off)")
    ap.add_argument("--worlds", type=int, default=0,
                    help="world count of the batch_worlds (default 4096) and diff_batch (default 1024) workloads")
    ap.add_argument("--threads", type=int, default=0, help="host threads of the batch_worlds workload (0: 4 per core)")
    ap.add_argument("--start-step", type=int, default=-1,
                    help="untimed steps before the warm-up (default: per workload)")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)
    if args.workload == "diff_batch" and "--steps" not in sys.argv:
        args.steps = 120
    if args.start_step < 0:
        args.start_step = START_STEPS[args.workload]

    rank = int(os.environ.get("RANK", "0"))
    world_size = int(os.environ.get("WORLD_SIZE", "1"))
    kind, a, b, c, seed, flags, desc = WORKLOADS[args.workload]
    config = {"workload": args.workload, "description": desc, "dt": 1.0 / 60.0, "substeps": 4,
              "timed_window": f"steps {args.start_step + args.warmup + 1}..{args.start_step + args.warmup + args.steps}",
              "continuous": not bool(flags & B.NO_CONTINUOUS), "sleep": False,
              "l2": "flushed between timed steps (256 MiB write, outside the timed region)",
              "parallelism": f"replicas x{args.gpus}" if args.gpus > 1 else "single world"}

    if args.worlds <= 0:
        args.worlds = 1024 if args.workload == "diff_batch" else 4096
    if args.impl == "reference":
        if rank != 0:
            return
        batched = args.workload in ("batch_worlds", "diff_batch")
        impl = cpu_impl()
        if batched:
            r = run_cpu_batch(args, 60.0, args.steps, impl)
            sample = f"{r['steps']} steps of {r['worlds']} worlds after {args.warmup} untimed steps"
        else:
            r = run_cpu_sample(args, budget_s=60.0, max_steps=args.steps, impl=impl)
            sample = f"{r['steps']} steps after {args.start_step + args.warmup} untimed steps"
        cores = r["threads"]
        sample += ", " + cpu_description(impl, cores, batched)
        line = {"metric": "body-steps/s", "value": r["value"], "unit": "body-steps/s", "n_gpus": args.gpus,
                "steps": r["steps"], "warmup": args.warmup, "ms_per_step": 1e3 * r["seconds"] / max(1, r["steps"]),
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic (seeded scene builders)", "config": config, "impl": "reference",
                "cpu_baseline": {"value": r["value"], "unit": "body-steps/s", "cores": cores, "kind": impl,
                                 "sample": sample,
                                 "library": str(REF_LIB.relative_to(ROOT)) if impl == "reference" else
                                 str(ORACLE_LIB.relative_to(ROOT))},
                "e2e": {"value": r["value"], "unit": "body-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return

    if args.workload == "diff_batch" and args.impl == "gb300":
        if rank != 0:
            return
        r = run_diff(args)
        total_s = r["fwd_s"] + r["bwd_s"]
        value = r["dyn"] * args.steps / total_s
        pk = peaks()
        achieved = r["tape_bytes"] / (r["adj_ms"] * 1e-3) / 1e9 if r["adj_ms"] > 0 else 0.0
        cpu = None
        if not args.no_cpu_baseline:
            impl = cpu_impl()
            c = run_cpu_batch(args, 20.0, args.steps, impl)
            cpu = {"value": c["value"], "unit": "body-steps/s (forward only: the reference has no adjoint)",
                   "cores": c["threads"], "kind": impl,
                   "sample": f"{c['steps']} forward steps of {c['worlds']} ramp worlds, "
                             + cpu_description(impl, c["threads"], True)}
        config.update({"worlds": args.worlds, "host_threads": r["threads"], "steps_per_pass": args.steps,
                       "l2": "inputs larger than L2 (every world's tape), no flush",
                       "timing": "wall clock of the forward pass (recording) and of the adjoint through the public API"})
        line = {
            "metric": "body-steps/s", "value": value, "unit": "body-steps/s (forward + adjoint)", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total_s / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded scene builders)", "config": config,
            "forward": {"seconds": r["fwd_s"], "value": r["dyn"] * args.steps / r["fwd_s"],
                        "without_recording_seconds": r["plain_s"], "batch_ms_per_step": r["profile"]},
            "adjoint": {"seconds": r["bwd_s"], "device_ms": r["adj_ms"], "over_forward": r["bwd_s"] / r["fwd_s"],
                        "gradients_finite": r["finite"]},
            "roofline": {"bound": "hbm", "kernel": "k_adjointStep", "achieved": achieved, "peak": pk["hbm_gbs"],
                         "unit": "GB/s", "frac": achieved / pk["hbm_gbs"], "peak_source": pk["source"], "traffic": None,
                         "alg_bytes": r["tape_bytes"], "note": "tape bytes read once by the adjoint / its device time"},
            "cpu_baseline": cpu,
            "e2e": {"value": value, "unit": "body-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0,
                    "read": "final centers of mass and the gradients, through the public API"},
            "gpu_launches": r["launches"], "clocks": r["clocks"],
        }
        print(json.dumps(line))
        return

    if args.workload == "batch_worlds" and args.impl == "gb300":
        if rank != 0:
            return
        r = run_batch(args)
        r["cpu"] = None
        r["pose_error"] = None
        if not args.no_cpu_baseline:
            impl = cpu_impl()
            c = run_cpu_batch(args, 20.0, args.steps, impl, gpu_states=r["states"])
            r["cpu"] = {"value": c["value"], "unit": "body-steps/s", "cores": c["threads"], "kind": impl,
                        "sample": f"{c['steps']} steps of {c['worlds']} worlds after {args.warmup} untimed steps, "
                                  + cpu_description(impl, c["threads"], True)}
            r["pose_error"] = c["pose_error"]
        value = r["dyn"] * args.steps / r["batch_s"]
        plain = r["dyn"] * r["plain_steps"] / r["plain_s"]
        config.update({"worlds": args.worlds, "host_threads": r["threads"],
                       "l2": "inputs larger than L2 (all worlds' state and constraints), no flush",
                       "timing": "wall clock; each world's step returns after its device work completes"})
        line = {
            "metric": "body-steps/s", "value": value, "unit": "body-steps/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * r["batch_s"] / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded scene builders)",
            "config": config, "plain_loop": {"value": plain, "steps": r["plain_steps"], "speedup": value / plain},
            "roofline": None, "cpu_baseline": r["cpu"],
            "pose_error": r["pose_error"] and dict(r["pose_error"], against=r["cpu"]["kind"],
                                                   after_steps=args.warmup + args.steps),
            "e2e": {"value": r["e2e_value"], "unit": "body-steps/s", "h2d_bytes_per_step": r["h2d"],
                    "d2h_bytes_per_step": r["d2h"], "read": "every world's move events after every batched step"},
            "gpu_launches": r["launches"], "clocks": r["clocks"],
            "batch_ms_per_step": r["profile"], "host_cpu_ms_per_step": r["host_cpu_ms"],
        }
        print(json.dumps(line))
        return

    if world_size > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    r = run_gpu(args, rank, world_size)
    total_ms = r["total_ms"]
    if world_size > 1:
        import torch
        import torch.distributed as dist

        t = torch.tensor([total_ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
    if rank != 0:
        return
    value = world_size * r["dyn"] * args.steps / (total_ms * 1e-3)
    cpu = port = err = None
    if not args.no_cpu_baseline:
        impl = cpu_impl()
        c = run_cpu_sample(args, budget_s=20.0, max_steps=400, impl=impl, gpu_state=r["window_state"])
        cpu = {"value": c["value"], "unit": "body-steps/s", "cores": c["threads"], "kind": impl,
               "sample": f"{c['steps']} steps ({c['seconds']:.1f} s) of the same world after "
                         f"{args.start_step + args.warmup} untimed steps, " + cpu_description(impl, c["threads"], False)}
        err = c["pose_error"] and dict(c["pose_error"], against=impl)
        if impl == "reference":
            o = run_cpu_sample(args, budget_s=10.0, max_steps=400, impl="port", gpu_state=r["window_state"])
            port = {"value": o["value"], "unit": "body-steps/s", "cores": o["threads"], "kind": "port",
                    "sample": f"{o['steps']} steps ({o['seconds']:.1f} s), " + cpu_description("port", o["threads"], False),
                    "pose_error": o["pose_error"]}
    pk = r["peak"]
    line = {
        "metric": "body-steps/s", "value": value, "unit": "body-steps/s", "n_gpus": world_size, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded scene builders)", "config": config,
        "roofline": {"bound": "hbm", "kernel": "solver (prepare..store)", "achieved": r["achieved_gbs"],
                     "peak": pk["hbm_gbs"], "unit": "GB/s", "frac": r["achieved_gbs"] / pk["hbm_gbs"],
                     "peak_source": pk["source"], "traffic": SOLVER_TRAFFIC.get(args.workload),
                     "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of the solver-stage kernels per "
                                       "step, timed steps (profiles/solver_traffic_timed_steps.md)",
                     "alg_bytes_per_step": r["alg_bytes"] / args.steps,
                     "solver_ms_per_step": r["solver_ms"] / args.steps},
        "cpu_baseline": cpu,
        "cpu_port": port,
        "pose_error": err,
        "e2e": {"value": r["e2e_value"] * world_size, "unit": "body-steps/s", "h2d_bytes_per_step": r["e2e_h2d"],
                "d2h_bytes_per_step": r["e2e_d2h"], "step_ms": r["e2e_step_ms"], "read_ms": r["e2e_read_ms"],
                "read": "b2World_GetBodyEvents after every step (transforms of all awake bodies)"},
        "gpu_launches": r["launches"],
        "clocks": r["clocks"],
        "stage_ms_per_step": [x / args.steps for x in r["stage_ms"]],
        "host_ms_per_step": {k: v / args.steps for k, v in zip(HOST_PHASES, r["host_ms"])},
    }
    print(json.dumps(line))


if __name__ == "__main__":
    main()
