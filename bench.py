"""Benchmark of the GB300 DPD engine: bead-steps/s of the FP32 batched engine on the
512-state grid against the plain one-state-at-a-time FP64 engine, with the served stream's
p50/p99 job latency and the 128^3 HBM-roofline run beside it.

Workload (default, `batched512`): 512 independent polymer-solvent states, cube side uniform
on 8..32 (17,880,960 beads in total), types W/H/T, 5% of the beads in H-T-T-T-T-T chains
(Hookean k=128 r0=0.5, angle k=20 theta0=0), a_WW=a_HH=a_TT=25, a_WH=35, a_WT ~ U[25,100]
and gamma ~ U[3,6] per state, dt=0.01, state seed = index + 1.  Synthetic data: seeded uniform
positions, Gaussian kT=1 velocities.  A "step" is one DPD timestep of every state.  The
grid's bead payload (~1 GB) is larger than L2, so no flush is needed.

  value     FP32 bead-steps/s of the whole grid resident on the GPU (one arena, one brick work
            queue, each step one CUDA-graph replay, autotuned kernel): K steps timed with CUDA
            events on the engine's stream, barrier + synchronize on both sides.
  e2e       the same metric through the C ABI with host buffers: AttachBatch (upload of the
            512 states) + Run(K) + read-back of x, v, f of every state, timed on the host.
  plain_fp64  the plain FP64 engine run one state at a time (Attach excluded, as the
            reference's bpsExec), and the batched / plain ratio.
  roofline  the force pass (bond kernel + brick kernel, dominant): algorithmic bytes per launch
            (1,180 B per bead-step x beads) / its average CUDA-event duration, against the
            measured HBM copy bandwidth.
  roofline_run  the 128^3 box (6,291,456 beads, same chain recipe, a_WT = 75, gamma = 4.5):
            value, e2e, roofline and phases of the single large state.
  serving   the served stream (Poisson arrivals at 50 jobs/s for 20 s, continuous batching):
            p50/p99 latency, served bead-steps/s over the whole run and at steady state (while
            the stream arrives, after a 2 s ramp; with the fractions of that time the GPU
            stepped and the host re-packed), served / offered, and against sequential
            execution.  The offered load exceeds the server's capacity, so a queue builds and
            the latencies measure it.
  serving_light  the same job mix at 20 jobs/s for 10 s, below capacity: latency without a
            standing queue.
  cpu_baseline  the oracle (C restatement of the reference's FP64 half-step engine) on all
            host cores, on a bounded sample of the same workload, with the host's CPU and,
            beside it, the reference's own TBB engine's expected rate: the port's rate times
            the reference/port ratio measured with both on one host (oracle/ref/calibrate.py;
            the reference sources are not present where this runs).

--workload polymer128 (or polymer32, water8) makes the single box the headline instead.
--impl reference times the reference's CPU implementation of the path (the oracle port;
the reference sources are not present where this runs) on a bounded sample of the same
workload and metric.
"""

from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "poets-dpd_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import numpy as np  # noqa: E402

import pdpd_world as W  # noqa: E402

ALGO_BYTES = {"fp32": 1180.0, "fp64": 2188.0}  # per bead-step, half-shell cell-list stream model
COMPULSORY_BYTES = 88.0
FALLBACK_HBM_GBS = 6800.0

WORKLOADS = {
    # name: (box side, chain fraction, seed, dt)
    "polymer128": (128, 0.05, 3, 0.01),
    "polymer32": (32, 0.10, 2, 0.01),
    "water8": (8, 0.0, 1, 0.02),
}
GRID = "batched512"          # the 512-state grid (pdpd_world.make_batched_grid)
GRID_STATES = 512
REF_SAMPLE_BEADS = 200_000   # the CPU sample of the grid: its first states up to this size


def make_world(name, side=None):
    L, frac, seed, dt = WORKLOADS[name]
    L = side or L
    if frac == 0.0:
        return W.make_water(L, seed=seed, dt=dt)
    return W.make_polymer_box(L, chain_fraction=frac, seed=seed, dt=dt)


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    return FALLBACK_HBM_GBS, "fallback"


class ClockSampler:
    """nvidia-smi clock / throttle samples during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index=0):
        self.device_index = device_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device_index), f"--query-gpu={self.QUERY}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
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
        return False

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
            for nm, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)),
                "reasons": sorted(reasons), "samples": len(sm)}


def oracle_rate(world, max_seconds=12.0, max_steps=200, threads=None):
    """Oracle (C port of the reference's FP64 half-step engine) bead-steps/s on all host
    cores: runs steps until max_seconds or max_steps."""
    import oracle as O

    threads = threads or os.cpu_count() or 1
    ow = O.OracleWorld(world)
    ow.run(1, nthreads=threads)  # warm-up
    steps, t0 = 0, time.perf_counter()
    while steps < max_steps and time.perf_counter() - t0 < max_seconds:
        ow.run(1, nthreads=threads)
        steps += 1
    dt = time.perf_counter() - t0
    return world.n_beads * steps / dt, threads, steps, dt


CALIBRATION = os.path.join(ROOT, "oracle", "tbb_calibration.json")


def host_cpu():
    """The host CPU as lscpu reports it: model, threads, SMT (threads per core), cores."""
    info = {"threads": os.cpu_count() or 1}
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
    except (OSError, subprocess.TimeoutExpired):
        return info
    keys = {"Model name": "model", "Thread(s) per core": "smt", "Core(s) per socket":
            "cores_per_socket", "Socket(s)": "sockets", "Architecture": "arch"}
    for line in out.splitlines():
        k, _, v = line.partition(":")
        if k.strip() in keys and keys[k.strip()] not in info:
            v = v.strip()
            info[keys[k.strip()]] = int(v) if v.isdigit() else v
    return info


def reference_estimate(port_rate, sample_key):
    """The reference's own TBB engine's expected rate on the same sample and cores: the port's
    measured rate times the reference/port ratio that oracle/ref/calibrate.py measured with
    both on one host (the reference sources exist only where that ran)."""
    if not os.path.exists(CALIBRATION):
        return None
    with open(CALIBRATION) as fh:
        cal = json.load(fh)
    s = cal["samples"].get(sample_key)
    if not s:
        return None
    r = float(s["ratio_reference_over_port"])
    return {"value": port_rate * r, "unit": "bead-steps/s", "ratio_reference_over_port": r,
            "reference_engines": s["reference_engines"],
            "calibrated_on": f"{cal['host'].get('model', '?')}, {cal['threads']} threads "
                             f"({cal['host'].get('machine', '?')}), {cal['when']}",
            "note": "estimate: the port's rate measured here x the ratio measured with both "
                    "engines on the calibration host"}


def calibration_key(workload):
    """The calibration sample of a workload's CPU sample (oracle/tbb_calibration.json)."""
    return {GRID: "grid3", "polymer128": "polymer32", "polymer32": "polymer32"}.get(workload)


def grid_sample(n_states=GRID_STATES, min_beads=REF_SAMPLE_BEADS):
    """The grid's first states, as many as reach min_beads (the same states every run)."""
    worlds = []
    for w in W.make_batched_grid(n_states, count=16):
        worlds.append(w)
        if sum(x.n_beads for x in worlds) >= min_beads:
            break
    return worlds


def oracle_rate_multi(worlds, max_seconds=12.0, max_steps=200, threads=None):
    """Oracle bead-steps/s on all host cores over several states: a step is one step of
    every state in turn; runs steps until max_seconds or max_steps."""
    import oracle as O

    threads = threads or os.cpu_count() or 1
    ows = [O.OracleWorld(w) for w in worlds]
    for ow in ows:
        ow.run(1, nthreads=threads)  # warm-up
    steps, t0 = 0, time.perf_counter()
    while steps < max_steps and time.perf_counter() - t0 < max_seconds:
        for ow in ows:
            ow.run(1, nthreads=threads)
        steps += 1
    dt = time.perf_counter() - t0
    return sum(w.n_beads for w in worlds) * steps / dt, threads, steps, dt


def batched_fp64_metrics(worlds, steps=10, device=0):
    """All states on one FP64 engine (the bit-exact precision, batched): the like-for-like
    counterpart of the FP32 headline, CUDA events around the run on the engine's stream."""
    import torch

    import pdpd_engine as E

    dev = torch.device("cuda", device)
    total = sum(w.n_beads for w in worlds)
    e64 = E.GB300DPDEngine("fp64", device=device)
    s64 = torch.cuda.ExternalStream(e64.stream(), device=dev)
    e64.AttachBatch([w.copy() for w in worlds])
    e64.run_async(3)
    e64.sync()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(s64)
    e64.run_async(steps)
    b.record(s64)
    e64.sync()
    torch.cuda.synchronize()
    ms = a.elapsed_time(b)
    e64.close()
    return {"value": total * steps / (ms / 1e3), "unit": "bead-steps/s", "steps": steps,
            "note": "every state attached to one FP64 engine (bit-exact with the reference), "
                    "stepped together"}


def plain_fp64_metrics(worlds, plain_steps=10, device=0):
    """The plain FP64 engine run one state at a time (Attach excluded from the time, as the
    reference's bpsExec), `plain_steps` steps per state, CUDA events around each Run."""
    import torch

    import pdpd_engine as E

    dev = torch.device("cuda", device)
    total = sum(w.n_beads for w in worlds)
    e64 = E.GB300DPDEngine("fp64", device=device)
    s64 = torch.cuda.ExternalStream(e64.stream(), device=dev)
    ms_total = 0.0
    for w in worlds:
        e64.Attach(w.copy())
        e64.run_async(2)
        e64.sync()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(s64)
        e64.run_async(plain_steps)
        b.record(s64)
        e64.sync()
        torch.cuda.synchronize()
        ms_total += a.elapsed_time(b)
    e64.close()
    return {"value": total * plain_steps / (ms_total / 1e3), "unit": "bead-steps/s",
            "steps_per_state": plain_steps,
            "note": "FP64 engine (bit-exact with the reference), one state at a time, "
                    "Attach excluded"}


def serving_metrics(rate=50.0, window_s=4.0, budget=40 << 30, interval=100, seed=5, device=0,
                    seq_fp32=16, seq_fp64=4):
    """Serving stream: Poisson arrivals at `rate` jobs/s for `window_s` seconds (seeded).  Each
    job is pure DPD water (density 3, a = 25, gamma = 4.5, dt = 0.02) in a cube of side
    log-uniform on [8, 64] (rounded), n_steps uniform on 100..2000, a host callback every
    `interval` steps, `budget` bytes of admission budget.  A client thread submits each job at
    its arrival time to the FP32 job server (continuous batching).  Served bead-steps/s = all
    jobs' bead-steps / (first arrival -> last completion); latency = arrival -> final callback.
    Sequential: a seeded sample of the same jobs run one at a time on the plain engines (Attach
    + Run(intervals, callback) + the remainder, the reference's pattern), wall clock per job."""

    import pdpd_engine as E

    rng = np.random.default_rng(seed)
    arrivals = []
    t = rng.exponential(1.0 / rate)
    while t < window_s:
        arrivals.append(t)
        t += rng.exponential(1.0 / rate)
    sides = np.clip(np.rint(8.0 * 8.0 ** rng.uniform(size=len(arrivals))), 8, 64).astype(int)
    nsteps = rng.integers(100, 2001, size=len(arrivals))
    worlds = [W.make_water(int(L), seed=k + 1, gen_seed=10_000 + k) for k, L in enumerate(sides)]
    total_bs = int(sum(w.n_beads * int(n) for w, n in zip(worlds, nsteps)))

    srv = E.GB300DPDServer("fp32", device=device, memory_budget_bytes=budget,
                           interval_steps=interval, keep_results=False)
    srv.submit(W.make_water(8, seed=1), 2 * interval)  # warm-up: module load, first graph
    srv.drain()
    st0 = srv.stats()
    launches0 = srv.kernel_launches()
    t0 = time.perf_counter()

    def client():
        for a, w, n in zip(arrivals, worlds, nsteps):
            d = t0 + a - time.perf_counter()
            if d > 0:
                time.sleep(d)
            srv.submit(w, int(n))

    th = threading.Thread(target=client)
    th.start()
    # the server's counters every 0.25 s while the stream arrives (steady_state)
    samples = []
    while th.is_alive():
        s_ = srv.stats()
        samples.append((time.perf_counter() - t0, s_["bead_steps"] - st0["bead_steps"],
                        s_["step_s"] - st0["step_s"], s_["repack_s"] - st0["repack_s"],
                        s_["host_gap_s"] - st0["host_gap_s"]))
        th.join(0.25)
    srv.drain()
    wall = time.perf_counter() - t0
    st = srv.stats()
    launches = srv.kernel_launches() - launches0
    srv.close()
    served = (st["bead_steps"] - st0["bead_steps"]) / wall

    pick = np.random.default_rng(seed + 1).permutation(len(worlds))

    def sequential(prec, count):
        eng = E.GB300DPDEngine(prec, device=device)
        eng.Attach(W.make_water(8, seed=1))
        eng.Run(interval)
        bs, secs = 0, 0.0
        for k in pick[:count]:
            w, n = worlds[k].copy(), int(nsteps[k])
            t1 = time.perf_counter()
            eng.Attach(w)
            eng.Run(n // interval, interval, lambda: True)
            if n % interval:
                eng.Run(n % interval)
            secs += time.perf_counter() - t1
            bs += w.n_beads * n
        eng.close()
        return bs / secs, count

    seq32, n32 = sequential("fp32", seq_fp32) if seq_fp32 else (None, 0)
    seq64, n64 = sequential("fp64", seq_fp64) if seq_fp64 else (None, 0)
    steady = steady_state(samples, ramp_s=min(2.0, window_s / 4), end_s=window_s)
    offered = total_bs / window_s
    return {"workload": f"Poisson {rate:g} jobs/s for {window_s:g} s ({len(worlds)} jobs), water "
                        f"sides log-uniform 8..64, n_steps U{{100..2000}}, callback every "
                        f"{interval} steps, {budget / 2**30:g} GiB budget",
            "jobs": len(worlds), "offered_bead_steps_per_s": offered,
            "served_bead_steps_per_s": served, "served_over_offered": served / offered,
            "steady_state": steady, "wall_s": wall,
            "latency_p50_s": st["latency_p50_s"], "latency_p99_s": st["latency_p99_s"],
            "latency_max_s": st["latency_max_s"], "max_active_jobs": st["max_active"],
            "repacks": st["repacks"] - st0["repacks"],
            "repack_s": st["repack_s"] - st0["repack_s"],
            "wasted_bead_steps": st["wasted_bead_steps"] - st0["wasted_bead_steps"],
            "step_s": st["step_s"] - st0["step_s"],
            "host_gap_s": st["host_gap_s"] - st0["host_gap_s"],
            "callback_s": st["callback_s"] - st0["callback_s"],
            "epochs": st["epochs"] - st0["epochs"],
            "between_epochs_s": st["between_s"] - st0["between_s"],
            "copy_wait_s": st["copy_wait_s"] - st0["copy_wait_s"],
            "sync_wait_s": st["sync_wait_s"] - st0["sync_wait_s"],
            "snap_alloc_s": st["snap_alloc_s"] - st0["snap_alloc_s"],
            "post_launch_s": st["post_launch_s"] - st0["post_launch_s"],
            "gpu_launches": launches,
            "sequential_fp32_bead_steps_per_s": seq32, "sequential_fp32_sample_jobs": n32,
            "sequential_fp64_bead_steps_per_s": seq64, "sequential_fp64_sample_jobs": n64,
            "served_vs_sequential_fp32": served / seq32 if seq32 else None,
            "served_vs_sequential_fp64": served / seq64 if seq64 else None,
            "steady_vs_sequential_fp32": steady["served_bead_steps_per_s"] / seq32
            if seq32 and steady else None}


def steady_state(samples, ramp_s, end_s):
    """Served rate while the stream arrives, after the ramp: from the server's counters sampled
    over time, (t, bead_steps, step_s, repack_s[, host_gap_s]), the slope between the first
    sample at or after ramp_s and the last at or before end_s, and the fractions of that wall
    time the GPU spent stepping (device time of the epochs), the host spent re-packing, and
    the GPU waited for the host between epochs (re-packs included)."""
    win = [x for x in samples if ramp_s <= x[0] <= end_s]
    if len(win) < 2 or win[-1][0] <= win[0][0]:
        return None
    a, b = win[0], win[-1]
    dt = b[0] - a[0]
    out = {"from_s": a[0], "to_s": b[0], "served_bead_steps_per_s": (b[1] - a[1]) / dt,
           "step_frac": (b[2] - a[2]) / dt, "repack_frac": (b[3] - a[3]) / dt,
           "bead_steps_per_step_s": (b[1] - a[1]) / (b[2] - a[2]) if b[2] > a[2] else None}
    if len(a) > 4:
        out["host_gap_frac"] = (b[4] - a[4]) / dt
    return out


def dist_setup(n_gpus):
    """One process per GPU under torchrun: (rank, world_size, local rank).  Replicas only: the
    ranks exchange nothing but the barrier and the max-over-ranks time (NCCL on GPUs, gloo
    where there is no GPU, e.g. the CPU tests of this path)."""
    rank, world_size = int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1))
    if world_size > 1:
        import torch
        import torch.distributed as dist

        local = int(os.environ.get("LOCAL_RANK", rank))
        if not dist.is_initialized():
            if torch.cuda.is_available():
                torch.cuda.set_device(local)
                dist.init_process_group("nccl")
            else:
                dist.init_process_group("gloo")
        return rank, world_size, local
    return 0, 1, 0


def max_over_ranks(x: float, world_size: int) -> float:
    """The largest of the ranks' values (the job's time is its slowest replica's)."""
    if world_size <= 1:
        return float(x)
    import torch
    import torch.distributed as dist

    dev = torch.device("cuda", torch.cuda.current_device()) if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.barrier()
    return float(t.item())


def aggregate_rate(units_per_rank: float, ms: float, world_size: int) -> float:
    """Whole-job throughput: every rank processed units_per_rank in at most ms."""
    return world_size * units_per_rank / (ms / 1e3)


def run_reference_arm(args):
    """The reference's CPU implementation of the path (the oracle port) on a bounded sample of
    the workload, all host cores; rank 0 only (the other ranks exit without work)."""
    rank, world_size, _ = dist_setup(args.gpus)
    if rank != 0:
        return
    import oracle as O

    if args.workload == GRID:
        worlds = grid_sample()
        workload = grid_workload_name(GRID_STATES)
        sample = (f"the grid's first {len(worlds)} states ({sum(w.n_beads for w in worlds)} "
                  f"beads), one step of each per step")
    else:
        worlds = [make_world(args.workload, side=args.ref_side)]
        L = WORKLOADS[args.workload][0]
        workload = f"{args.workload}: {L}^3 polymer-solvent box recipe"
        sample = f"{args.ref_side}^3 box of the same recipe ({worlds[0].n_beads} beads)"
    threads = os.cpu_count() or 1
    ows = [O.OracleWorld(w) for w in worlds]
    for _ in range(args.warmup):
        for ow in ows:
            ow.run(1, nthreads=threads)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        for ow in ows:
            ow.run(1, nthreads=threads)
    dt = time.perf_counter() - t0
    rate = sum(w.n_beads for w in worlds) * args.steps / dt
    line = {
        "impl": "reference", "metric": METRIC, "value": rate, "unit": "bead-steps/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * dt / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": workload, "sample": sample, "parallelism": "replicas only"},
        "cpu_baseline": {"value": rate, "unit": "bead-steps/s", "cores": threads, "kind": "port",
                         "sample": f"{sample}, {args.steps} steps", "host": host_cpu(),
                         "reference_tbb_estimate": reference_estimate(
                             rate, calibration_key(args.workload))},
        "e2e": {"value": rate, "unit": "bead-steps/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def grid_workload_name(n_states):
    part = "" if n_states == GRID_STATES else f" (its first {n_states})"
    return (f"{GRID}: {GRID_STATES} polymer-solvent states{part}, sides U{{8..32}}, density 3, "
            f"5% H-T5 chains, a_WT ~ U[25,100], gamma ~ U[3,6], fp32 batched")


def upload_bytes(worlds, fp64=False):
    """Host-to-device bytes of an Attach: x, v, f (doubles) and the hash of every bead, the
    flat bond lists (bead ids) and a parameter row per bond and angle (the per-bead bond
    tables are built on the device)."""
    total = 0
    for w in worlds:
        n = w.n_beads
        bb, _, _, ab, _, _ = w.flat_bonds()
        total += (n * (9 * 8 + 4) + (2 * bb.shape[0] + 3 * ab.shape[0]) * 4
                  + (bb.shape[0] + ab.shape[0]) * (32 if fp64 else 16))
    return total


def host_link_gbs(device, nbytes=1 << 30):
    """Pinned-memory DMA bandwidth of the host link each way (GB/s, best of 3 under CUDA
    events): the floor under the e2e run's uploads and read-backs."""
    import torch

    h = torch.empty(nbytes, dtype=torch.uint8, pin_memory=True)
    d = torch.empty(nbytes, dtype=torch.uint8, device=device)
    out = {}
    for name, (dst, src) in (("h2d", (d, h)), ("d2h", (h, d))):
        dst.copy_(src, non_blocking=True)
        torch.cuda.synchronize()
        best = float("inf")
        for _ in range(3):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            dst.copy_(src, non_blocking=True)
            e1.record()
            e1.synchronize()
            best = min(best, e0.elapsed_time(e1))
        out[name] = nbytes / best / 1e6
    del h, d
    return out


def e2e_phases(eng, worlds, steps):
    """Where an e2e run's wall time goes, from a second run of the same calls split at their
    boundaries (wall clock, ms): AttachBatch of the host worlds (the Python binding's
    flattening included), the K steps (run_async + sync), and the read-back of every state
    into its host arrays."""
    t0 = time.perf_counter()
    eng.AttachBatch(worlds)
    t1 = time.perf_counter()
    eng.run_async(steps)
    eng.sync()
    t2 = time.perf_counter()
    eng.read_states(into=worlds)
    t3 = time.perf_counter()
    return {"attach": 1e3 * (t1 - t0), "steps": 1e3 * (t2 - t1), "read_back": 1e3 * (t3 - t2)}


def e2e_floor(e2e, steps, ms_per_step, link):
    """The e2e rate if the uploads and read-backs ran at the link's DMA bandwidth and nothing
    else cost time beside the K steps: adds link, copy_floor_ms, floor and frac_of_floor."""
    copy_ms = (e2e["h2d_bytes_per_step"] * steps / link["h2d"] + e2e["d2h_bytes_per_step"] * steps / link["d2h"]) / 1e6
    bead_steps = e2e["value"] * e2e["wall_s"]
    floor = bead_steps / ((steps * ms_per_step + copy_ms) / 1e3)
    e2e.update({"link_gbs": link, "copy_floor_ms": copy_ms, "floor": floor, "frac_of_floor": e2e["value"] / floor})
    return e2e


ISSUE_SLOTS_PER_S = 152 * 4 * 2.07e9  # warp-instruction issue slots per second of a GB300


def force_roofline(phases, beads, precision, traffic_key=None):
    """Roofline of the force pass from profile_run's per-phase CUDA-event times; traffic from
    the ncu capture summarised in profiles/force_kernel_traffic.json (per bead-step)."""
    force_ms = phases["force_ms"] / max(1, phases["force_launches"])
    peak, peak_kind = measured_peaks()
    achieved = ALGO_BYTES[precision] * beads / (force_ms / 1e3) / 1e9
    traffic = instr = pipes = None
    tpath = os.path.join(ROOT, "profiles", "force_kernel_traffic.json")
    if os.path.exists(tpath):
        with open(tpath) as fh:
            tj = json.load(fh)
        key = traffic_key or precision
        if f"{key}_bytes_per_bead_step" in tj:
            traffic = tj[f"{key}_bytes_per_bead_step"] * beads
        if f"{key}_warp_instructions_per_bead_step" in tj:
            instr = tj[f"{key}_warp_instructions_per_bead_step"]
        pipes = tj.get(f"{key}_pipes")
    roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "traffic": traffic, "kernel": "force", "kernel_ms": force_ms,
            "algo_bytes_per_bead_step": ALGO_BYTES[precision], "peak_source": peak_kind,
            "compulsory_frac": COMPULSORY_BYTES * beads / (force_ms / 1e3) / 1e9 / peak}
    if traffic is not None:
        # what the kernel really moves: its ncu DRAM bytes over the same time
        roof["dram_gbs"] = traffic / (force_ms / 1e3) / 1e9
        roof["dram_frac"] = roof["dram_gbs"] / peak
    if instr is not None:
        # the bound that applies: one warp instruction per SMSP per clock
        # (GB300: 152 SMs x 4 SMSPs x 2.07 GHz), the kernel's ncu instructions per bead
        cap = ISSUE_SLOTS_PER_S
        roof["issue"] = {"warp_instructions_per_bead_step": instr, "slots_per_s": cap,
                         "frac": instr * beads / (force_ms / 1e3) / cap}
    if pipes is not None:
        # FP32 (FMA) and integer (ALU) pipe utilisation of the kernel, from its ncu capture
        roof["pipes"] = dict(pipes, source="ncu --set full of one launch (profiles/)")
    ph = {"force": force_ms, "sort": phases["sort_ms"] / max(1, phases["sort_launches"])}
    return roof, ph


def kernel_config(eng):
    return {k: v for k, _, v in eng.GetConfigEntries()
            if k in ("force_kernel", "brick_x", "brick_y", "brick_z", "autotune")}


def host_copies(eng):
    """How the attach and the read-backs moved the beads: "direct" (a kernel reading and
    writing the host arrays over the host link) or "staged" (pinned buffers and DMA)."""
    v = {k: v for k, _, v in eng.GetConfigEntries()}.get("host_direct", "0")
    return "direct" if v == "1" else "staged"


def fixed_kernel(eng, args):
    """--force-kernel K: run FP32 force kernel K (no autotuning), for profiling a variant;
    --host-direct 0: the host copies through pinned staging and DMA, to measure that path."""
    if args.force_kernel:
        eng.SetConfigEntry("force_kernel", args.force_kernel)
    if args.host_direct is not None:
        eng.SetConfigEntry("host_direct", args.host_direct)


def tune(eng, attach, steps=64):
    """Autotune once (its trials are ordinary steps: the trajectory does not depend on the
    choice), then keep the chosen kernel and brick shape fixed."""
    eng.SetConfigEntry("autotune", 1)
    attach()
    eng.run_async(steps)
    eng.sync()
    tuned = {k: v for k, _, v in eng.GetConfigEntries()}
    eng.SetConfigEntry("autotune", 0)
    # keep the pick: configured entries are not replaced by the size-aware default
    for k in ("force_kernel", "brick_x", "brick_y", "brick_z"):
        eng.SetConfigEntry(k, int(tuned[k]))
    return {k: tuned.get(k) for k in ("force_kernel", "brick_x", "brick_y", "brick_z", "autotune")}


def timed_run(eng, steps, warmup, dev, local, world_size, attach):
    """Resident-state rate: attach, warm up, then `steps` graph replays between CUDA events on
    the engine's stream (barrier + synchronize on both sides), clocks sampled meanwhile."""
    import torch

    attach()
    eng.run_async(warmup)
    eng.sync()
    stream = torch.cuda.ExternalStream(eng.stream(), device=dev)
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    if world_size > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    launches0 = eng.kernel_launches()
    with ClockSampler(local) as clocks:
        time.sleep(0.3)
        ev0.record(stream)
        eng.run_async(steps)
        ev1.record(stream)
        eng.sync()
        torch.cuda.synchronize()
        time.sleep(0.2)
    launches = eng.kernel_launches() - launches0
    ms = max_over_ranks(ev0.elapsed_time(ev1), world_size)
    return ms, launches, clocks.summary()


def measure_grid(args, dev, local, world_size):
    """The headline: the 512-state grid on one FP32 engine."""
    import pdpd_engine as E

    n_states = args.grid_states
    worlds = W.make_batched_grid(GRID_STATES, count=n_states)
    total = sum(w.n_beads for w in worlds)
    eng = E.GB300DPDEngine("fp32", device=local)
    fixed_kernel(eng, args)
    tuned = (tune(eng, lambda: eng.AttachBatch([w.copy() for w in worlds]))
             if args.autotune and not args.force_kernel else None)
    # e2e: AttachBatch (upload) + Run(K) + read-back of every state, host buffers
    eng.AttachBatch([w.copy() for w in worlds])
    eng.Run(args.warmup)
    hw = [w.copy() for w in worlds]
    t0 = time.perf_counter()
    eng.AttachBatch(hw)
    eng.Run(args.steps)  # Run() reads x, v, f of every state back into the host worlds
    e2e_dt = time.perf_counter() - t0
    e2e = {"value": total * args.steps / e2e_dt, "unit": "bead-steps/s", "wall_s": e2e_dt,
           "h2d_bytes_per_step": upload_bytes(worlds) / args.steps,
           "d2h_bytes_per_step": total * 72 / args.steps,
           "host_copies": host_copies(eng),
           "note": "AttachBatch (upload of all states) + Run(K) + read-back of x, v, f of every "
                   "state; bytes are per step of K"}
    ms, launches, clocks = timed_run(eng, args.steps, args.warmup, dev, local, world_size,
                                     lambda: eng.AttachBatch([w.copy() for w in worlds]))
    if tuned is None:  # the size-aware default the engine chose for this batch
        tuned = kernel_config(eng)
    e2e["phases_ms"] = e2e_phases(eng, [w.copy() for w in worlds], args.steps)
    e2e_floor(e2e, args.steps, ms / args.steps, host_link_gbs(dev))
    roof, ph = force_roofline(eng.profile_run(args.steps), total, "fp32", "fp32_grid")
    eng.close()
    plain = plain_fp64_metrics(worlds, device=local) if not args.no_plain and world_size == 1 else None
    value = aggregate_rate(total * args.steps, ms, world_size)
    if plain:
        plain["batched_vs_plain"] = value / world_size / plain["value"]
        plain["batched_fp64"] = batched_fp64_metrics(worlds, device=local)
        plain["batched_fp64_vs_plain"] = plain["batched_fp64"]["value"] / plain["value"]
    return {"value": value, "ms": ms, "beads": total, "e2e": e2e, "launches": launches,
            "clocks": clocks, "roofline": roof, "phases": ph, "tuned": tuned, "plain_fp64": plain,
            "config": {"workload": grid_workload_name(n_states), "states": n_states,
                       "beads": total, "precision": "fp32",
                       "l2": "state > L2 (no flush)",
                       "parallelism": "replicas only" if world_size > 1 else "single GPU"}}


def measure_box(args, name, side, precision, dev, local, world_size, autotune, snapshot=True):
    """One large state (the 128^3 HBM-roofline run by default)."""
    import pdpd_engine as E

    world = make_world(name, side=side)
    n = world.n_beads
    eng = E.GB300DPDEngine(precision, device=local)
    if precision == "fp32":
        fixed_kernel(eng, args)
    tuned = (tune(eng, lambda: eng.Attach(world.copy()))
             if precision == "fp32" and autotune and not args.force_kernel else None)
    # e2e: through the C ABI with host buffers (Attach = upload, Run, read-back)
    eng.Attach(world.copy())
    eng.Run(args.warmup)
    w_e2e = world.copy()
    t0 = time.perf_counter()
    eng.Attach(w_e2e)
    eng.Run(args.steps)  # Run() reads x, v, f back into the host world
    e2e_dt = time.perf_counter() - t0
    e2e = {"value": n * args.steps / e2e_dt, "unit": "bead-steps/s", "wall_s": e2e_dt,
           "h2d_bytes_per_step": upload_bytes([world], precision == "fp64") / args.steps,
           "d2h_bytes_per_step": n * 72 / args.steps, "host_copies": host_copies(eng),
           "note": "Attach (upload) + Run(K) + read-back of x, v, f; bytes are per step of K"}
    ms, launches, clocks = timed_run(eng, args.steps, args.warmup, dev, local, world_size,
                                     lambda: eng.Attach(world.copy()))
    if tuned is None:  # the size-aware default the engine chose for this world
        tuned = kernel_config(eng)
    e2e["phases_ms"] = e2e_phases(eng, [world.copy()], args.steps)
    e2e_floor(e2e, args.steps, ms / args.steps, host_link_gbs(dev))
    roof, ph = force_roofline(eng.profile_run(args.steps), n, precision)
    snap = None
    if snapshot and world_size == 1:
        # interval snapshots: the v2binary section encoded on the GPU vs the full read-back
        sec_bytes = eng.v2binary_prepare()
        eng.v2binary_encode()
        eng.read_state(0)
        reps = 3
        t0 = time.perf_counter()
        for _ in range(reps):
            eng.v2binary_encode()
        t_v2 = (time.perf_counter() - t0) / reps
        t0 = time.perf_counter()
        for _ in range(reps):
            eng.read_state(0)
        t_rs = (time.perf_counter() - t0) / reps
        snap = {"v2binary_bytes_per_bead": sec_bytes / n, "v2binary_ms": 1e3 * t_v2,
                "read_state_bytes_per_bead": 72.0, "read_state_ms": 1e3 * t_rs,
                "note": f"one snapshot of the {side or WORKLOADS[name][0]}^3 box: GPU-encoded "
                        f"v2binary section vs x, v, f read back as doubles (wall clock, host "
                        f"buffers)"}
    eng.close()
    L = side or WORKLOADS[name][0]
    return {"value": aggregate_rate(n * args.steps, ms, world_size), "ms": ms, "beads": n,
            "e2e": e2e, "launches": launches, "clocks": clocks, "roofline": roof, "phases": ph,
            "tuned": tuned, "snapshot": snap,
            "config": {"workload": f"{name}: {L}^3 box, density 3, {n} beads, "
                                   f"{WORKLOADS[name][1]:.0%} H-T5 chains, {precision}",
                       "beads": n, "precision": precision, "l2": "state > L2 (no flush)",
                       "parallelism": "replicas only" if world_size > 1 else "single GPU"}}


def run_engine_arm(args):
    import torch

    rank, world_size, local = dist_setup(args.gpus)
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    grid = args.workload == GRID
    if grid:
        main = measure_grid(args, dev, local, world_size)
        side = None
        if not args.no_roofline_run:
            side = measure_box(args, "polymer128", args.side, "fp32", dev, local, world_size,
                               args.autotune)
    else:
        main = measure_box(args, args.workload, args.side, args.precision, dev, local, world_size,
                           args.autotune)
        side = None
    serving = serving_light = None
    if args.serving_window > 0 and world_size == 1:
        serving = serving_metrics(window_s=args.serving_window, device=local)
    if args.serving_light_rate > 0 and args.serving_light_window > 0 and args.serving_window > 0 and world_size == 1:
        # the same job mix offered below the server's capacity: latency without a standing queue
        serving_light = serving_metrics(rate=args.serving_light_rate, window_s=args.serving_light_window,
                                        seed=6, device=local, seq_fp32=0, seq_fp64=0)
    if rank != 0:
        return
    cpu = None
    if not args.no_cpu_baseline:
        if grid:
            sample = grid_sample()
            rate, threads, steps, dt = oracle_rate_multi(sample)
            desc = (f"the grid's first {len(sample)} states ({sum(w.n_beads for w in sample)} "
                    f"beads), {steps} steps of each in {dt:.1f} s")
        else:
            rate, threads, steps, dt = oracle_rate(make_world(args.workload, side=args.ref_side))
            desc = f"{args.ref_side}^3 box of the same recipe, {steps} steps in {dt:.1f} s"
        cpu = {"value": rate, "unit": "bead-steps/s", "cores": threads, "kind": "port",
               "sample": desc, "host": host_cpu(),
               "reference_tbb_estimate": reference_estimate(rate, calibration_key(args.workload))}
    line = {
        "metric": METRIC, "value": main["value"], "unit": "bead-steps/s", "n_gpus": world_size,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": main["ms"] / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32" if (grid or args.precision == "fp32") else "f64", "data": "synthetic",
        "config": main["config"],
        "e2e": main["e2e"],
        "roofline": main["roofline"],
        "phases_ms_per_step": main["phases"],
        "clocks": main["clocks"],
        "gpu_launches": main["launches"],
        "cpu_baseline": cpu,
        "plain_fp64": main.get("plain_fp64"),
        "serving": serving,
        "serving_light": serving_light,
        "roofline_run": None if side is None else {
            "workload": side["config"]["workload"], "value": side["value"],
            "ms_per_step": side["ms"] / args.steps, "e2e": side["e2e"],
            "roofline": side["roofline"], "phases_ms_per_step": side["phases"],
            "clocks": side["clocks"], "gpu_launches": side["launches"],
            "kernel_config": side["tuned"]},
        "snapshot": (side or main).get("snapshot"),
        "kernel_config": main["tuned"],
    }
    print(json.dumps(line), flush=True)


METRIC = "bead-steps/s on 1 GB300 (FP32 batched vs plain FP64); served p50/p99 job latency"


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=500)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default=GRID, choices=[GRID] + sorted(WORKLOADS))
    ap.add_argument("--precision", default="fp32", choices=["fp32", "fp64"],
                    help="precision of a single-box workload (the grid is FP32)")
    ap.add_argument("--ref-side", type=int, default=32,
                    help="box side of the bounded CPU sample of a single-box workload")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-plain", action="store_true",
                    help="skip the plain FP64 state-by-state run of the grid")
    ap.add_argument("--no-roofline-run", action="store_true",
                    help="skip the 128^3 single-box run beside the grid")
    ap.add_argument("--autotune", type=int, default=1,
                    help="1: autotune the FP32 force kernel first (default); 0: default kernel")
    ap.add_argument("--force-kernel", type=int, default=0,
                    help="FP32 force kernel variant to run instead of autotuning (1, 6, 8, 9)")
    ap.add_argument("--host-direct", type=int, default=None, choices=[0, 1],
                    help="the engines' host_direct config (default: the engine's own, direct "
                         "where the device reaches host memory)")
    ap.add_argument("--serving-window", type=float, default=20.0,
                    help="seconds of Poisson arrivals of the serving stream (0 skips it)")
    ap.add_argument("--serving-light-rate", type=float, default=20.0,
                    help="jobs/s of a second stream below capacity (0 skips it)")
    ap.add_argument("--serving-light-window", type=float, default=10.0,
                    help="seconds of Poisson arrivals of the stream below capacity")
    ap.add_argument("--grid-states", type=int, default=GRID_STATES,
                    help="run the grid's first N states only (profiling on a smaller grid)")
    ap.add_argument("--side", type=int, default=None,
                    help="override the box side of the single-box run (profiling on smaller boxes)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference_arm(args)
    else:
        run_engine_arm(args)


if __name__ == "__main__":
    main()
