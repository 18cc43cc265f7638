"""The oracle (C restatement of the reference's half-step engine) is pinned bit for bit to
the reference's own outputs stored in tests/golden/ (generated by make_golden.py from the
reference's NaiveDPDEngineHalfStep, compiled unchanged)."""

import numpy as np
import pytest

import oracle as O
import pdpd_world as W
from _helpers import (load_hash_kat, load_world_fixture, merge_fixture_names, state_rel_err,
                      world_fixture_names)


def test_hash_known_answers_match_reference():
    kat = load_hash_kat()
    th, h, u = O.hash_batch(kat["t"], kat["seed"], kat["a"], kat["b"])
    assert np.array_equal(th, kat["t_hash"])
    assert np.array_equal(h, kat["h"])
    assert np.array_equal(u.view(np.uint32), kat["u"].view(np.uint32))


def test_hash_is_symmetric_and_in_range():
    kat = load_hash_kat()
    _, h1, u1 = O.hash_batch(kat["t"], kat["seed"], kat["a"], kat["b"])
    _, h2, _ = O.hash_batch(kat["t"], kat["seed"], kat["b"], kat["a"])
    assert np.array_equal(h1, h2)
    assert np.all(u1 >= -0.5) and np.all(u1 < 0.5)


@pytest.mark.parametrize("name", world_fixture_names())
@pytest.mark.parametrize("nthreads", [1, 3])
def test_oracle_bit_exact_vs_reference(name, nthreads):
    world, ref = load_world_fixture(name)
    ow = O.OracleWorld(world)
    prev = 0
    for k, c in enumerate(ref["checkpoints"]):
        ow.run(int(c) - prev, nthreads=nthreads)
        prev = int(c)
        assert ow.t == ref["t"][k]
        assert np.array_equal(ow.x, ref["x"][k]), f"{name}: x differs at step {c}"
        assert np.array_equal(ow.v, ref["v"][k]), f"{name}: v differs at step {c}"
        assert np.array_equal(ow.f, ref["f"][k]), f"{name}: f differs at step {c}"


def test_oracle_cell_index_is_floor():
    w = W.make_polymer_box(6, chain_fraction=0.1, seed=3)
    ow = O.OracleWorld(w)
    c = ow.cell_index()
    fl = np.floor(w.x).astype(np.int64)
    L = w.box.astype(np.int64)
    assert np.array_equal(c, fl[:, 0] * L[1] * L[2] + fl[:, 1] * L[2] + fl[:, 2])


def test_oracle_reports_snapped_bond():
    b = W.WorldBuilder((6, 6, 6), 1, [[25.0]], [[4.5]], dt=0.01)
    b.add_polymer_type([0, 0], [(0, 1, 128.0, 0.5)])
    b.add_polymer(0, [(1.0, 1.0, 1.0), (3.5, 1.0, 1.0)])
    ow = O.OracleWorld(b.build())
    with pytest.raises(RuntimeError, match="snapped"):
        ow.run(1)


def test_observables_basic():
    w = W.make_water(6, seed=1)
    ow = O.OracleWorld(w)
    obs = ow.observe(n_bins=20, n_bond_bins=10)
    assert abs(obs["ke2"] - np.sum(w.v ** 2)) < 1e-9 * obs["ke2"]
    assert np.allclose(obs["momentum"], 0, atol=1e-9)
    n = w.n_beads
    # every unordered pair with r < 1 counted once: expected count ~ N * rho * (4/3 pi) / 2
    pairs = obs["rdf"].sum()
    assert 0.7 * n * 3 * 4.18879 / 2 < pairs < 1.3 * n * 3 * 4.18879 / 2


def test_oracle_replays_reference_testbase_suite():
    """All 225 cases of the reference's own engine test suite, segment by segment: from the
    identical input state, the oracle reproduces the reference engine's output bit for bit."""
    from _helpers import load_testbase, world_at
    cases = load_testbase()
    assert len(cases) == 225
    n_seg = 0
    for name, world, segs in cases:
        for todo, t_in, s_in, t_out, s_out in segs:
            ow = O.OracleWorld(world_at(world, t_in, s_in))
            ow.run(todo)
            assert ow.t == t_out, name
            assert np.array_equal(np.hstack([ow.x, ow.v, ow.f]), s_out), name
            n_seg += 1
    assert n_seg == 900


@pytest.mark.parametrize("name", merge_fixture_names("stationary"))
def test_oracle_stationary_types_vs_reference_half_merge(name):
    """Stationary bead types against the reference's half-merge engine (the reference engine
    family member that supports them): stationary beads stay exactly where they are with v and
    f exactly zero after every step; every other bead agrees to summation-order roundoff."""
    world, ref = load_world_fixture(name)
    st = np.asarray(world.stationary, bool)[world.bead_type]
    assert st.any() and (~st).any()
    ow = O.OracleWorld(world)
    prev = 0
    for k, c in enumerate(ref["checkpoints"]):
        ow.run(int(c) - prev, nthreads=4)
        prev = int(c)
        assert ow.t == ref["t"][k]
        assert np.array_equal(ow.x[st], world.x[st]) and np.array_equal(ref["x"][k][st], world.x[st])
        assert not ow.v[st].any() and not ow.f[st].any()
        assert not ref["v"][k][st].any() and not ref["f"][k][st].any()
        assert np.max(np.abs(ow.x - ref["x"][k])) < 1e-12
        assert state_rel_err(ow.v, ref["v"][k]) < 1e-12
        assert state_rel_err(ow.f, ref["f"][k]) < 1e-12


@pytest.mark.parametrize("name", merge_fixture_names("spatial"))
def test_oracle_spatial_strengths_vs_reference_half_merge(name):
    """Spatially varying interaction strengths (Parameter expressions over the cell position),
    evaluated per cell by the reference, against the reference's half-merge engine: the pair
    strength is the mean of the two beads' cell values; agreement to summation-order
    roundoff."""
    world, ref = load_world_fixture(name)
    assert world.cell_conservative is not None
    ow = O.OracleWorld(world)
    plain = O.OracleWorld(world.copy())
    plain.cell_a = plain.cell_g = None  # the constant matrices: must differ (the test bites)
    prev = 0
    for k, c in enumerate(ref["checkpoints"]):
        ow.run(int(c) - prev, nthreads=4)
        prev = int(c)
        assert ow.t == ref["t"][k]
        assert np.max(np.abs(ow.x - ref["x"][k])) < 1e-12
        assert state_rel_err(ow.v, ref["v"][k]) < 1e-12
        assert state_rel_err(ow.f, ref["f"][k]) < 1e-12
    plain.run(int(ref["checkpoints"][0]))
    assert state_rel_err(plain.f, ref["f"][0]) > 1e-6
