"""Times the reference's own TBB CPU engines beside the oracle port, on the same sample and
the same cores, and records the ratio in oracle/tbb_calibration.json.

Baseline infrastructure: the reference sources exist only in the build container, so the
reference engine cannot run where the GPU numbers are taken.  There, bench.py times the
oracle port (oracle/pdpd_oracle.c) and scales it by the ratio recorded here to report the
reference engine's expected rate beside it.

    make -C oracle/ref all        # builds oracle/_ref/ref_tbb_bench (reference + TBB stand-in)
    python oracle/ref/calibrate.py

Samples (the ones bench.py's CPU leg times):
  grid3       the 512-state grid's first states up to 200,000 beads (one step of each per
              step); the reference engine per state is half_merge_tbb when all sides are
              multiples of 4, else half_step_tbb (naive_dpd_engine_half_merge.hpp:47-57);
  polymer32   the 32^3 polymer-solvent box (98,304 beads, 10% H-T5 chains), half_merge_tbb.
Each engine is first checked to reproduce the oracle's trajectory over 10 steps (the TBB
stand-in must not change what the engine computes); then both are timed with all host
threads: the reference as its benchmark_engine.cpp does (Run(k), k x1.5 until the rate is
stable within 5%), the port as bench.py does.
"""

from __future__ import annotations

import json
import os
import platform
import subprocess
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE = os.path.dirname(HERE)
ROOT = os.path.dirname(ORACLE)
sys.path.insert(0, os.path.join(ROOT, "poets-dpd_gb300"))
sys.path.insert(0, ORACLE)
sys.path.insert(0, ROOT)

import oracle as O  # noqa: E402
import pdpd_world as W  # noqa: E402

EXE = os.path.join(ORACLE, "_ref", "ref_tbb_bench")
OUT = os.path.join(ORACLE, "tbb_calibration.json")


def host_description():
    info = {"machine": platform.machine(), "threads": os.cpu_count()}
    try:
        lscpu = subprocess.run(["lscpu"], capture_output=True, text=True).stdout
        for line in lscpu.splitlines():
            k, _, v = line.partition(":")
            v = v.strip()
            if k == "Model name":
                info["model"] = v
            elif k == "Thread(s) per core":
                info["smt"] = int(v)
            elif k == "Core(s) per socket":
                info["cores_per_socket"] = int(v)
            elif k == "Socket(s)":
                info["sockets"] = int(v)
    except OSError:
        pass
    return info


def check_trajectory(world, path, tmp):
    """The reference TBB engine (through the stand-in) and the oracle agree over 10 steps."""
    out = os.path.join(tmp, "check.bin")
    subprocess.run([EXE, "check", "auto", path, "10", out], check=True,
                   stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
    raw = open(out, "rb").read()
    t = np.frombuffer(raw[:8], np.int64)[0]
    rec = np.frombuffer(raw[8:], np.float64).reshape(-1, 9)
    ow = O.OracleWorld(world)
    ow.run(10, nthreads=os.cpu_count())
    dx = np.abs(rec[:, 0:3] - ow.x)
    dx = np.minimum(dx, np.asarray(world.box, float)[None, :] - dx)
    err = float(dx.max())
    if t != world.t + 10 or not err < 1e-6:
        raise SystemExit(f"reference TBB engine disagrees with the oracle: t={t}, max|dx|={err}")
    return err


def time_reference(paths, threads, min_seconds):
    env = dict(os.environ, PDPD_NUM_THREADS=str(threads))
    r = subprocess.run([EXE, "auto", str(min_seconds), "4"] + paths, check=True,
                       capture_output=True, text=True, env=env)
    lines = [json.loads(x) for x in r.stdout.splitlines() if x.startswith("{")]
    return lines[-1]


def time_port(worlds, threads, max_seconds=12.0, max_steps=200):
    """The port as bench.py's CPU leg times it (oracle_rate_multi)."""
    ows = [O.OracleWorld(w) for w in worlds]
    for ow in ows:
        ow.run(1, nthreads=threads)
    steps, t0 = 0, time.perf_counter()
    while steps < max_steps and time.perf_counter() - t0 < max_seconds:
        for ow in ows:
            ow.run(1, nthreads=threads)
        steps += 1
    dt = time.perf_counter() - t0
    return sum(w.n_beads for w in worlds) * steps / dt, steps, dt


def main():
    import bench

    if not os.path.exists(EXE):
        raise SystemExit("build oracle/_ref/ref_tbb_bench first: make -C oracle/ref all")
    threads = os.cpu_count() or 1
    samples = {"grid3": bench.grid_sample(),
               "polymer32": [bench.make_world("polymer32")]}
    result = {"host": host_description(), "threads": threads,
              "when": time.strftime("%Y-%m-%dT%H:%M:%SZ", time.gmtime()),
              "reference_flags": "-O3 -ffast-math -DNDEBUG (reference makefile:38-39)",
              "port_flags": "-O2 -ffp-contract=off (oracle/Makefile)", "samples": {}}
    with tempfile.TemporaryDirectory() as tmp:
        for name, worlds in samples.items():
            paths = []
            for k, w in enumerate(worlds):
                p = os.path.join(tmp, f"{name}_{k}.pdw1")
                W.write_pdw1(w, p)
                paths.append(p)
            errs = [check_trajectory(w, p, tmp) for w, p in zip(worlds, paths)]
            ref = time_reference(paths, threads, min_seconds=10.0)
            port, steps, dt = time_port(worlds, threads)
            result["samples"][name] = {
                "beads": int(sum(w.n_beads for w in worlds)),
                "sides": [int(w.box[0]) for w in worlds],
                "reference_engines": ref["engines"],
                "reference_rate": ref["rate"], "reference_steps": ref["steps"],
                "port_rate": port, "port_steps": steps,
                "ratio_reference_over_port": ref["rate"] / port,
                "trajectory_check_max_dx": max(errs),
            }
            print(name, json.dumps(result["samples"][name]), flush=True)
    with open(OUT, "w") as f:
        json.dump(result, f, indent=1)
        f.write("\n")
    print("wrote", OUT)


if __name__ == "__main__":
    main()
