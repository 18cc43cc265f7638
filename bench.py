"""Benchmark of the GB300 DPD engine: bead-steps/s on the 128^3 polymer-solvent box.

Workload (default): 128x128x128 periodic box at density 3 = 6,291,456 beads, types W/H/T,
5% of the beads in H-T-T-T-T-T chains (Hookean k=128 r0=0.5, angle k=20 theta0=0),
a_WW=a_HH=a_TT=25, a_WH=35, a_WT=a_HT=75, gamma=4.5, dt=0.01, FP32 engine.  Synthetic data:
seeded uniform positions, Gaussian kT=1 velocities.  A "step" is one DPD timestep of the
whole box.  The state (~300 MB of bead payload) is larger than L2, so no flush is needed.

  value     bead-steps/s with the state resident on the GPU: K steps timed with CUDA events
            on the engine's stream (graph replays), barrier + synchronize on both sides.
  e2e       the same metric through the C ABI with host buffers: Attach (upload) + Run(K) +
            read back x, v, f, timed on the host.
  roofline  the force kernel (dominant): algorithmic bytes per launch (1,180 B per
            bead-step x beads) / its average CUDA-event duration, against the measured HBM
            copy bandwidth.
  cpu_baseline  the oracle (C restatement of the reference's FP64 half-step engine) on all
            host cores, on a bounded sample of the same recipe.

--impl reference times the reference's CPU implementation of the path (the oracle port;
the reference sources are not present where this runs) on the same recipe and metric.
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


def batched_grid_metrics(steps=200, plain_steps=10, n_states=512, device=0):
    """512 independent polymer-solvent states, cube side uniform on 8..32, per-state
    a_WT ~ U[25,100] and gamma ~ U[3,6], 5% chains, dt = 0.01, seeds = index + 1.

    FP32 batched: all states attached to one engine (one arena, one brick work queue over all
    states, each step one CUDA-graph replay), autotuned, `steps` steps timed with CUDA events.
    FP64 plain: the FP64 engine run one state at a time (Attach excluded from the time, as the
    reference's bpsExec), `plain_steps` steps per state, CUDA events around each Run."""
    import torch

    import pdpd_engine as E

    worlds = W.make_batched_grid(n_states)
    total = sum(w.n_beads for w in worlds)
    dev = torch.device("cuda", device)
    eng = E.GB300DPDEngine("fp32", device=device)
    eng.SetConfigEntry("autotune", 1)
    eng.AttachBatch([w.copy() for w in worlds])
    eng.run_async(40)  # the autotuner's trials are the first of these steps
    eng.sync()
    stream = torch.cuda.ExternalStream(eng.stream(), device=dev)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    ev0.record(stream)
    eng.run_async(steps)
    ev1.record(stream)
    eng.sync()
    torch.cuda.synchronize()
    batched = total * steps / (ev0.elapsed_time(ev1) / 1e3)
    tuned = {n: v for n, _, v in eng.GetConfigEntries()}
    eng.close()

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
    plain = total * plain_steps / (ms_total / 1e3)
    e64.close()
    return {"workload": f"{n_states} states, sides 8..32, {total} beads, 5% H-T5 chains",
            "beads": total, "fp32_batched": batched, "fp64_plain_state_by_state": plain,
            "ratio": batched / plain, "steps": steps, "plain_steps_per_state": plain_steps,
            "autotuned": {k: tuned[k] for k in ("force_kernel", "brick_x", "brick_y", "brick_z",
                                                "autotune")}}


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
    th.join()
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

    seq32, n32 = sequential("fp32", seq_fp32)
    seq64, n64 = sequential("fp64", seq_fp64)
    return {"workload": f"Poisson {rate:g} jobs/s for {window_s:g} s ({len(worlds)} jobs), water "
                        f"sides log-uniform 8..64, n_steps U{{100..2000}}, callback every "
                        f"{interval} steps, {budget / 2**30:g} GiB budget",
            "jobs": len(worlds), "offered_bead_steps_per_s": total_bs / window_s,
            "served_bead_steps_per_s": served, "wall_s": wall,
            "latency_p50_s": st["latency_p50_s"], "latency_p99_s": st["latency_p99_s"],
            "latency_max_s": st["latency_max_s"], "max_active_jobs": st["max_active"],
            "repacks": st["repacks"] - st0["repacks"],
            "repack_s": st["repack_s"] - st0["repack_s"],
            "wasted_bead_steps": st["wasted_bead_steps"] - st0["wasted_bead_steps"],
            "gpu_launches": launches,
            "sequential_fp32_bead_steps_per_s": seq32, "sequential_fp32_sample_jobs": n32,
            "sequential_fp64_bead_steps_per_s": seq64, "sequential_fp64_sample_jobs": n64,
            "served_vs_sequential_fp32": served / seq32, "served_vs_sequential_fp64": served / seq64}


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
    rank, world_size, _ = dist_setup(args.gpus)
    if rank != 0:
        return
    side = args.ref_side
    world = make_world(args.workload, side=side)
    import oracle as O

    threads = os.cpu_count() or 1
    ow = O.OracleWorld(world)
    for _ in range(args.warmup):
        ow.run(1, nthreads=threads)
    t0 = time.perf_counter()
    ow.run(args.steps, nthreads=threads)
    dt = time.perf_counter() - t0
    rate = world.n_beads * args.steps / dt
    L = WORKLOADS[args.workload][0]
    line = {
        "impl": "reference", "metric": "bead-steps/s", "value": rate, "unit": "bead-steps/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * dt / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"{args.workload}: {L}^3 polymer-solvent box recipe",
                   "sample": f"{side}^3 box of the same recipe ({world.n_beads} beads)",
                   "parallelism": "replicas only"},
        "cpu_baseline": {"value": rate, "unit": "bead-steps/s", "cores": threads, "kind": "port",
                         "sample": f"{side}^3 box, {world.n_beads} beads, {args.steps} steps"},
        "e2e": {"value": rate, "unit": "bead-steps/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_engine_arm(args):
    import torch

    import pdpd_engine as E

    rank, world_size, local = dist_setup(args.gpus)
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    world = make_world(args.workload, side=args.side)
    n = world.n_beads
    eng = E.GB300DPDEngine(args.precision, device=local)

    # --- autotune once (its trials are ordinary steps: the trajectory does not depend on the
    # choice), then fix the chosen kernel and brick shape for every measurement below
    if args.precision == "fp32" and args.autotune:
        eng.SetConfigEntry("autotune", 1)
        eng.Attach(world.copy())
        eng.run_async(64)
        eng.sync()
        tuned = {k: v for k, _, v in eng.GetConfigEntries()}
        eng.SetConfigEntry("autotune", 0)
    else:
        tuned = {k: v for k, _, v in eng.GetConfigEntries()}

    # --- e2e: through the C ABI with host buffers (Attach = upload, Run, read-back)
    w_e2e = world.copy()
    eng.Attach(w_e2e)
    eng.Run(args.warmup)
    torch.cuda.synchronize()
    w_e2e = world.copy()
    t0 = time.perf_counter()
    eng.Attach(w_e2e)
    eng.Run(args.steps)  # Run() reads x, v, f back into the host world
    e2e_dt = time.perf_counter() - t0
    h2d = n * (9 * 8 + 4)
    bb, _, _, ab, _, _ = w_e2e.flat_bonds()
    h2d += (n + 1) * 4 + (2 * bb.shape[0] + 3 * ab.shape[0]) * 16
    d2h = n * 9 * 8
    e2e_rate = n * args.steps / e2e_dt

    # --- value: resident state, graph replays, CUDA events on the engine's stream
    w = world.copy()
    eng.Attach(w)
    eng.run_async(args.warmup)
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
        eng.run_async(args.steps)
        ev1.record(stream)
        eng.sync()
        torch.cuda.synchronize()
        time.sleep(0.2)
    launches = eng.kernel_launches() - launches0
    ms = max_over_ranks(ev0.elapsed_time(ev1), world_size)
    value = aggregate_rate(n * args.steps, ms, world_size)

    # --- dominant kernel: per-phase CUDA-event times over the same number of steps
    phases = eng.profile_run(args.steps)

    # --- interval snapshots: the v2binary section encoded on the GPU vs the full read-back
    snapshot = None
    if world_size == 1 and args.precision in ("fp32", "fp64"):
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
        snapshot = {"v2binary_bytes_per_bead": sec_bytes / n, "v2binary_ms": 1e3 * t_v2,
                    "read_state_bytes_per_bead": 72.0, "read_state_ms": 1e3 * t_rs,
                    "note": "one snapshot of the whole box: GPU-encoded v2binary section vs x, v, f "
                            "read back as doubles (wall clock, host buffers)"}
    force_ms = phases["force_ms"] / max(1, phases["force_launches"])
    peak, peak_kind = measured_peaks()
    algo = ALGO_BYTES[args.precision] * n
    achieved = algo / (force_ms / 1e3) / 1e9
    traffic = None
    tpath = os.path.join(ROOT, "profiles", "force_kernel_traffic.json")
    if os.path.exists(tpath):
        with open(tpath) as fh:
            tj = json.load(fh)
        key = f"{args.precision}_bytes_per_bead_step"
        if key in tj:
            traffic = tj[key] * n

    batched = None
    if not args.no_batched and world_size == 1:
        batched = batched_grid_metrics(device=local)
    serving = None
    if args.serving_window > 0 and world_size == 1:
        serving = serving_metrics(window_s=args.serving_window, device=local)
    if rank != 0:
        return
    cpu = None
    if not args.no_cpu_baseline:
        sample_side = args.ref_side
        rate, threads, steps, dt = oracle_rate(make_world(args.workload, side=sample_side))
        cpu = {"value": rate, "unit": "bead-steps/s", "cores": threads, "kind": "port",
               "sample": f"{sample_side}^3 box of the same recipe, {steps} steps in {dt:.1f} s"}
    L = args.side or WORKLOADS[args.workload][0]
    line = {
        "metric": "bead-steps/s", "value": value, "unit": "bead-steps/s", "n_gpus": world_size,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32" if args.precision == "fp32" else "f64", "data": "synthetic",
        "config": {"workload": f"{args.workload}: {L}^3 box, density 3, {n} beads, "
                               f"{WORKLOADS[args.workload][1]:.0%} H-T5 chains, {args.precision}",
                   "beads": n, "precision": args.precision, "l2": "state > L2 (no flush)",
                   "parallelism": "replicas only" if world_size > 1 else "single GPU"},
        "e2e": {"value": e2e_rate, "unit": "bead-steps/s", "h2d_bytes_per_step": h2d / args.steps,
                "d2h_bytes_per_step": d2h / args.steps,
                "note": "Attach (upload) + Run(K) + read-back of x, v, f; bytes are per step of K"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic,
                     "kernel": "force", "kernel_ms": force_ms,
                     "algo_bytes_per_bead_step": ALGO_BYTES[args.precision],
                     "peak_source": peak_kind,
                     "compulsory_frac": COMPULSORY_BYTES * n / (force_ms / 1e3) / 1e9 / peak},
        "phases_ms_per_step": {"force": force_ms,
                               "sort": phases["sort_ms"] / max(1, phases["sort_launches"])},
        "clocks": clocks.summary(),
        "gpu_launches": launches,
        "cpu_baseline": cpu,
        "batched_grid": batched,
        "serving": serving,
        "snapshot": snapshot,
        "kernel_config": {k: tuned.get(k) for k in ("force_kernel", "brick_x", "brick_y", "brick_z",
                                                    "autotune")},
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=500)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="polymer128", choices=sorted(WORKLOADS))
    ap.add_argument("--precision", default="fp32", choices=["fp32", "fp64"])
    ap.add_argument("--ref-side", type=int, default=32,
                    help="box side of the bounded CPU sample (same recipe)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batched", action="store_true",
                    help="skip the 512-state batched grid (FP32 batched vs FP64 plain)")
    ap.add_argument("--autotune", type=int, default=1,
                    help="1: autotune the FP32 force kernel first (default); 0: default kernel")
    ap.add_argument("--serving-window", type=float, default=4.0,
                    help="seconds of Poisson arrivals of the serving stream (0 skips it)")
    ap.add_argument("--side", type=int, default=None,
                    help="override the box side of the workload (profiling on smaller boxes)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference_arm(args)
    else:
        run_engine_arm(args)


if __name__ == "__main__":
    main()
