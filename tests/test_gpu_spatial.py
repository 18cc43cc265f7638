"""Spatially varying DPD parameters on the GPU.

The reference's half-merge engine supports interaction strengths that are expressions of the
cell position (naive_dpd_engine_half_merge.hpp:221-236: evaluated per cell at Attach; a pair
uses the mean of its two beads' cell values of a_ij and of sqrt(gamma_ij), :570-583).  The
fixtures tests/golden/merge_spatial_*.npz hold the per-cell values the reference evaluated and
its trajectory.  Tolerances as for the other half-merge fixtures: FP64 engine bit-exact with
the oracle and within 1e-12 of the reference (another summation order); FP32 one-step forces
within 1e-5.
"""

import numpy as np
import pytest

import oracle as O
import pdpd_engine as E
import pdpd_world as W
from _helpers import force_rel_err, load_world_fixture, merge_fixture_names, state_rel_err

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", merge_fixture_names("spatial"))
def test_fp64_spatial_bit_exact_vs_oracle_and_close_to_half_merge(name):
    world, ref = load_world_fixture(name)
    ow = O.OracleWorld(world)
    eng = E.GB300DPDEngine("fp64")
    w = world.copy()
    eng.Attach(w)
    prev = 0
    for k, c in enumerate(ref["checkpoints"]):
        eng.Run(int(c) - prev)
        ow.run(int(c) - prev, nthreads=8)
        prev = int(c)
        assert np.array_equal(w.x, ow.x) and np.array_equal(w.v, ow.v) and np.array_equal(w.f, ow.f)
        assert np.max(np.abs(w.x - ref["x"][k])) < 1e-12
        assert state_rel_err(w.v, ref["v"][k]) < 1e-12
        assert state_rel_err(w.f, ref["f"][k]) < 1e-12
    got = eng.observe(n_bins=20, n_bond_bins=20)
    obs = ow.observe(n_bins=20, n_bond_bins=20)
    assert got["virial"] == pytest.approx(obs["virial"], rel=1e-12)


@pytest.mark.parametrize("name", merge_fixture_names("spatial"))
@pytest.mark.parametrize("configured", [6, 9])
def test_fp32_spatial(name, configured):
    """The FP32 engine runs spatial worlds on the thread-per-bead kernel whatever kernel is
    configured; forces within the FP32 tolerance, trajectories identical across configs."""
    world, ref = load_world_fixture(name)
    eng = E.GB300DPDEngine("fp32")
    eng.SetConfigEntry("force_kernel", configured)
    w = world.copy()
    eng.Attach(w)
    eng.Run(1)
    assert force_rel_err(w.f, ref["f"][0]) <= 1e-5
    eng.Run(9)
    other = E.GB300DPDEngine("fp32")
    other.SetConfigEntry("force_kernel", 1)
    w2 = world.copy()
    other.Attach(w2)
    other.Run(10)
    assert np.array_equal(w.x, w2.x) and np.array_equal(w.v, w2.v)


def test_spatial_world_in_a_batch_equals_alone():
    world, _ = load_world_fixture("merge_spatial_polymer")
    plain = W.make_polymer_box(9, chain_fraction=0.1, seed=4)
    for prec in ("fp32", "fp64"):
        alone = [world.copy(), plain.copy()]
        for w in alone:
            e = E.GB300DPDEngine(prec)
            e.Attach(w)
            e.Run(12)
        pair = [plain.copy(), world.copy()]
        e2 = E.GB300DPDEngine(prec)
        e2.AttachBatch(pair)
        e2.Run(12)
        assert np.array_equal(pair[1].x, alone[0].x) and np.array_equal(pair[1].f, alone[0].f)
        # the plain world runs on the thread-per-bead kernel in this batch: bit-identical too
        assert np.array_equal(pair[0].x, alone[1].x) and np.array_equal(pair[0].f, alone[1].f)
