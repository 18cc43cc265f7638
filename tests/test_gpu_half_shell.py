"""The half-shell FP32 force kernel (force_kernel 9): each pair inside a brick is evaluated once
and its reaction passed to the other bead (Newton's third law, the forward half shell of the
reference's make_nhood.hpp:40-49 and naive_dpd_engine_half_merge.hpp:198-219).

Its pair force is exactly antisymmetric and the sums are integer, so its results do not depend
on which side evaluated a pair, on the order of the sums, on the brick shape or on the batch.
These tests check those properties bit for bit, its global-memory fallback, and its accuracy
against the oracle (the FP32 tolerance of the other kernels) over one and ten steps.
"""

import numpy as np
import pytest

import oracle as O
import pdpd_engine as E
import pdpd_world as W
from _helpers import force_rel_err, periodic_dx

pytestmark = pytest.mark.gpu

FP32_FORCE_TOL = 1e-5


def _run(world, steps, **cfg):
    w = world.copy()
    eng = E.GB300DPDEngine("fp32")
    eng.SetConfigEntry("force_kernel", 9)
    for k, v in cfg.items():
        eng.SetConfigEntry(k, v)
    eng.Attach(w)
    eng.Run(steps)
    return w


def _same(a, b):
    assert a.t == b.t
    assert np.array_equal(a.x, b.x) and np.array_equal(a.v, b.v) and np.array_equal(a.f, b.f)


def test_half_shell_polymer_box_vs_oracle_one_and_ten_steps():
    world = W.make_polymer_box(32, chain_fraction=0.1, seed=2)
    ow = O.OracleWorld(world)
    ow.run(1, nthreads=16)
    w = _run(world, 1)
    assert force_rel_err(w.f, ow.f) <= FP32_FORCE_TOL
    ow.run(9, nthreads=16)
    w10 = _run(world, 10)
    assert np.max(np.abs(periodic_dx(w10.x, ow.x, world.box))) < 1e-4
    assert np.max(np.abs(w10.v - ow.v)) < 1e-3


def test_half_shell_equals_full_shell_within_tolerance():
    """On the same state the half shell's forces are those of the full shell (variant 8) up to
    the order of the sums and the form of the separation (the full shell rounds o_i + 1 for a
    pair across a face in the -1 direction, 6e-8 absolute): far inside the FP32 tolerance."""
    world = W.make_polymer_box(24, chain_fraction=0.1, seed=12)
    half = _run(world, 1)
    full = world.copy()
    eng = E.GB300DPDEngine("fp32")
    eng.SetConfigEntry("force_kernel", 8)
    eng.Attach(full)
    eng.Run(1)
    assert np.array_equal(half.x, full.x)  # the first update_pos precedes any force
    assert force_rel_err(half.f, full.f) <= 3e-6


def test_half_shell_batch_equals_alone():
    """A world alone and inside a batch of other worlds (which changes the default brick
    shape and the work queue) gives the same state to the bit."""
    a = W.make_polymer_box(11, chain_fraction=0.1, seed=21)
    b = W.make_water((7, 13, 9), seed=22)
    c = W.make_polymer_box(17, chain_fraction=0.05, seed=23)
    alone = _run(a, 25)
    batch = [b.copy(), a.copy(), c.copy()]
    eng = E.GB300DPDEngine("fp32")
    eng.SetConfigEntry("force_kernel", 9)
    eng.AttachBatch(batch)
    eng.Run(25)
    _same(alone, batch[1])
    _same(_run(c, 25), batch[2])


def test_half_shell_overflow_fallback_is_bit_identical():
    """Half the beads packed into a 2x2x2-cell corner: bricks there do not fit in shared memory
    and take the global-memory path, whose fixed-point sums equal the staged half shell's."""
    w = W.make_water(8, seed=5, dt=0.005)
    rng = np.random.default_rng(7)
    half = w.n_beads // 2
    w.x[:half] = 3.0 + 2.0 * rng.random((half, 3))
    ref = _run(w, 3, brick_x=2, brick_y=2, brick_z=2)
    for shape in ((8, 8, 8), (4, 4, 8), (1, 1, 1)):
        _same(ref, _run(w, 3, brick_x=shape[0], brick_y=shape[1], brick_z=shape[2]))
    ow = O.OracleWorld(w)
    ow.run(1)
    assert force_rel_err(_run(w, 1).f, ow.f) <= FP32_FORCE_TOL


@pytest.mark.parametrize("side", [2, 3, 5])
def test_half_shell_small_periodic_boxes(side):
    """Boxes smaller than a brick's halo: a halo cell is a periodic image of a home cell, so a
    pair can be met at two images; each image is its own pair, as in the reference."""
    world = W.make_water(side, seed=30 + side)
    ow = O.OracleWorld(world)
    ow.run(1)
    assert force_rel_err(_run(world, 1).f, ow.f) <= FP32_FORCE_TOL
