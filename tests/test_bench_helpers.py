"""The bench's own arithmetic, on the CPU: the grid sample the CPU arms time, the upload byte
count of an attach and the roofline figures derived from per-phase device times."""

import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402
import pdpd_world as W  # noqa: E402


def test_grid_sample_is_the_grids_first_states():
    sample = bench.grid_sample()
    grid = W.make_batched_grid(bench.GRID_STATES, count=len(sample))
    assert [w.n_beads for w in sample] == [w.n_beads for w in grid]
    assert sum(w.n_beads for w in sample) >= bench.REF_SAMPLE_BEADS
    assert sum(w.n_beads for w in sample[:-1]) < bench.REF_SAMPLE_BEADS
    assert np.array_equal(sample[0].x, grid[0].x)


def test_upload_bytes_counts_state_hashes_and_bonds():
    w = W.make_polymer_box(8, chain_fraction=0.1, seed=3)
    bb, _, _, ab, _, _ = w.flat_bonds()
    n = w.n_beads
    lists = (2 * bb.shape[0] + 3 * ab.shape[0]) * 4
    expect = n * (9 * 8 + 4) + lists + (bb.shape[0] + ab.shape[0]) * 16
    assert bench.upload_bytes([w]) == expect
    assert bench.upload_bytes([w, w]) == 2 * expect
    assert bench.upload_bytes([w], fp64=True) == expect + (bb.shape[0] + ab.shape[0]) * 16


def test_e2e_floor_arithmetic():
    # 1e9 bead-steps in 2 s; K = 10 steps of 100 ms (1 s); 200 GB up at 200 GB/s (1 s) and
    # 100 GB down at 100 GB/s (1 s): a floor of 3 s
    e2e = {"value": 5e8, "wall_s": 2.0, "h2d_bytes_per_step": 20e9, "d2h_bytes_per_step": 10e9}
    out = bench.e2e_floor(e2e, 10, 100.0, {"h2d": 200.0, "d2h": 100.0})
    assert out["copy_floor_ms"] == pytest.approx(2000.0)
    assert out["floor"] == pytest.approx(1e9 / 3.0)
    assert out["frac_of_floor"] == pytest.approx(5e8 / (1e9 / 3.0))


def test_force_roofline_arithmetic():
    phases = {"force_ms": 20.0, "force_launches": 10, "sort_ms": 3.0, "sort_launches": 10}
    roof, ph = bench.force_roofline(phases, 1_000_000, "fp32")
    assert ph == {"force": 2.0, "sort": 0.3}
    assert roof["kernel_ms"] == 2.0
    assert roof["achieved"] == pytest.approx(1180.0 * 1e6 / 2e-3 / 1e9)
    assert roof["frac"] == pytest.approx(roof["achieved"] / roof["peak"])
    assert roof["bound"] == "hbm" and roof["unit"] == "GB/s"
    # beside the model: the kernel's ncu DRAM bytes and instructions per bead over the same time
    assert roof["dram_gbs"] == pytest.approx(roof["traffic"] / 2e-3 / 1e9)
    issue = roof["issue"]
    assert issue["frac"] == pytest.approx(issue["warp_instructions_per_bead_step"] * 1e6 / 2e-3 /
                                          bench.ISSUE_SLOTS_PER_S)


def test_grid_workload_name_names_the_grid():
    assert bench.grid_workload_name(512).startswith("batched512: 512 polymer-solvent states")
    assert "(its first 64)" in bench.grid_workload_name(64)


def test_steady_state_slope_of_the_server_counters():
    # (t, bead_steps, step_s, repack_s): 4e9 bead-steps/s from t = 2 on, the GPU stepping 90%
    # of the time and re-packing 2%; the ramp before t = 2 is left out
    samples = [(0.5 * k, (0 if k < 4 else 4e9 * (0.5 * k - 2.0)) + 1e6 * min(k, 4),
                0.45 * k, 0.01 * k) for k in range(41)]
    st = bench.steady_state(samples, ramp_s=2.0, end_s=15.0)
    assert st["from_s"] == 2.0 and st["to_s"] == 15.0
    assert st["served_bead_steps_per_s"] == pytest.approx(4e9)
    assert st["step_frac"] == pytest.approx(0.9)
    assert st["repack_frac"] == pytest.approx(0.02)
    assert bench.steady_state(samples[:3], ramp_s=2.0, end_s=15.0) is None
