"""Stationary bead types on the GPU.

The reference's half-step engine does not support them; its half-merge engine does
(naive_dpd_engine_half_merge.hpp:329-333 update_pos skipped, :387-394 v and f cleared,
:440-449 and :516-522 no force between two stationary beads).  The fixtures under
tests/golden/merge_*.npz were made by that engine.  Tolerances:
* FP64 engine: bit-exact with the oracle (the half-step order plus the stationary rules);
  against the half-merge engine, which adds the same terms in another order, x within 1e-12
  and v, f within 1e-12 relative.
* FP32 engine: one-step forces within 1e-5 relative (as every FP32 parity test).
* Stationary beads, both engines: v and f exactly zero after every step, position constant
  (FP64: bit-identical to the input; FP32: the input rounded to a cell + FP32 offset).
"""

import numpy as np
import pytest

import oracle as O
import pdpd_engine as E
import pdpd_world as W
from _helpers import force_rel_err, load_world_fixture, merge_fixture_names, state_rel_err

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", merge_fixture_names("stationary"))
def test_fp64_stationary_bit_exact_vs_oracle_and_close_to_half_merge(name):
    world, ref = load_world_fixture(name)
    st = np.asarray(world.stationary, bool)[world.bead_type]
    x0 = world.x.copy()
    ow = O.OracleWorld(world)
    eng = E.GB300DPDEngine("fp64")
    w = world.copy()
    eng.Attach(w)
    prev = 0
    for k, c in enumerate(ref["checkpoints"]):
        eng.Run(int(c) - prev)
        ow.run(int(c) - prev, nthreads=8)
        prev = int(c)
        assert w.t == ref["t"][k]
        assert np.array_equal(w.x, ow.x) and np.array_equal(w.v, ow.v) and np.array_equal(w.f, ow.f)
        assert np.array_equal(w.x[st], x0[st])
        assert not w.v[st].any() and not w.f[st].any()
        assert np.max(np.abs(w.x - ref["x"][k])) < 1e-12
        assert state_rel_err(w.v, ref["v"][k]) < 1e-12
        assert state_rel_err(w.f, ref["f"][k]) < 1e-12


@pytest.mark.parametrize("name", merge_fixture_names("stationary"))
@pytest.mark.parametrize("force_kernel", [6, 8, 9, 1])
def test_fp32_stationary(name, force_kernel):
    world, ref = load_world_fixture(name)
    st = np.asarray(world.stationary, bool)[world.bead_type]
    eng = E.GB300DPDEngine("fp32")
    eng.SetConfigEntry("force_kernel", force_kernel)
    w = world.copy()
    eng.Attach(w)
    eng.Run(1)
    assert force_rel_err(w.f, ref["f"][0]) <= 1e-5
    x1 = w.x.copy()
    assert np.max(np.abs(x1[st] - world.x[st])) < 1e-6
    for _ in range(3):
        eng.Run(5)
        assert np.array_equal(w.x[st], x1[st])
        assert not w.v[st].any() and not w.f[st].any()


def test_stationary_world_in_a_batch_equals_alone():
    world, _ = load_world_fixture("merge_stationary_anchor")
    other = W.make_polymer_box(9, chain_fraction=0.1, seed=4)
    for prec in ("fp32", "fp64"):
        alone = world.copy()
        e1 = E.GB300DPDEngine(prec)
        e1.Attach(alone)
        e1.Run(12)
        pair = [other.copy(), world.copy()]
        e2 = E.GB300DPDEngine(prec)
        e2.AttachBatch(pair)
        e2.Run(12)
        assert np.array_equal(pair[1].x, alone.x) and np.array_equal(pair[1].v, alone.v)
        assert np.array_equal(pair[1].f, alone.f)
