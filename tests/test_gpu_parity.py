"""GPU parity: the engine, called through its C ABI, against the reference's outputs
(tests/golden/, made by the reference's own FP64 engine) and against the oracle.

Tolerances:
* FP64 engine: bit-exact -- x, v, f identical to the reference / oracle after every
  checkpoint (same operation order, no fused multiply-add).
* RNG and bead-to-cell assignment: bit-exact.
* FP32 engine, one step from an FP64 state: max_i |f_i - f_ref_i| / rms|f_ref| <= 1e-5.
* FP32 engine, 10 steps: positions within 1e-4 and velocities within 1e-3 of the FP64
  reference (absolute, periodic distance); the reference's own differential test allows
  0.01*sqrt(steps) (test_differential.hpp:70-71).
"""

import numpy as np
import pytest

import oracle as O
import pdpd_engine as E
import pdpd_world as W
from _helpers import (force_rel_err, fp32_force_check, load_hash_kat, load_world_fixture, periodic_dx,
                      world_fixture_names)

pytestmark = pytest.mark.gpu

FP32_FORCE_TOL = 1e-5
FP32_X10_TOL = 1e-4
FP32_V10_TOL = 1e-3


def run_checkpoints(engine, world, checkpoints):
    engine.Attach(world)
    out = []
    prev = 0
    for c in checkpoints:
        engine.Run(int(c) - prev)
        prev = int(c)
        out.append((world.t, world.x.copy(), world.v.copy(), world.f.copy()))
    return out


# ---------------------------------------------------------------------------- RNG

def test_rng_bit_exact_vs_reference_kat():
    kat = load_hash_kat()
    h, u = E.rng_eval(kat["t"], kat["seed"], kat["a"], kat["b"])
    assert np.array_equal(h, kat["h"])
    assert np.array_equal(u.view(np.uint32), kat["u"].view(np.uint32))


def test_rng_bit_exact_vs_oracle_random():
    rng = np.random.default_rng(99)
    n = 1 << 22
    t = rng.integers(0, 2**32, n, dtype=np.uint64).astype(np.uint32)
    seed = rng.integers(0, 2**63, n, dtype=np.uint64)
    a = rng.integers(0, 2**32, n, dtype=np.uint64).astype(np.uint32)
    b = rng.integers(0, 2**32, n, dtype=np.uint64).astype(np.uint32)
    h, u = E.rng_eval(t, seed, a, b)
    _, h_ref, u_ref = O.hash_batch(t, seed, a, b)
    assert np.array_equal(h, h_ref)
    assert np.array_equal(u.view(np.uint32), u_ref.view(np.uint32))


# ---------------------------------------------------------------------------- FP64 bit-exact

@pytest.mark.parametrize("name", world_fixture_names())
def test_fp64_bit_exact_vs_reference(name):
    world, ref = load_world_fixture(name)
    eng = E.GB300DPDEngine("fp64")
    got = run_checkpoints(eng, world, ref["checkpoints"])
    for k, (t, x, v, f) in enumerate(got):
        c = ref["checkpoints"][k]
        assert t == ref["t"][k]
        assert np.array_equal(x, ref["x"][k]), f"{name}: x differs after {c} steps"
        assert np.array_equal(v, ref["v"][k]), f"{name}: v differs after {c} steps"
        assert np.array_equal(f, ref["f"][k]), f"{name}: f differs after {c} steps"


@pytest.mark.parametrize("L,steps", [(32, 10)])
def test_fp64_bit_exact_vs_oracle_polymer_box(L, steps):
    """32^3 polymer box (98,304 beads, 10% H-T5 chains), FP64 engine vs oracle."""
    world = W.make_polymer_box(L, chain_fraction=0.1, seed=2)
    ow = O.OracleWorld(world)
    eng = E.GB300DPDEngine("fp64")
    eng.Attach(world)
    for k in (1, steps - 1):
        eng.Run(k)
        ow.run(k, nthreads=16)
        assert np.array_equal(world.x, ow.x)
        assert np.array_equal(world.v, ow.v)
        assert np.array_equal(world.f, ow.f)


@pytest.fixture(scope="module")
def large_box_one_step():
    """The 128^3 polymer box of the HBM-roofline configuration (5% chains, seed 3; 6,291,456
    beads) and the oracle's state after one FP64 step from it (computed once for the FP64
    and FP32 tests)."""
    world = W.make_polymer_box(128, chain_fraction=0.05, seed=3)
    ow = O.OracleWorld(world)
    ow.run(1, nthreads=16)
    return world, ow


def test_fp64_bit_exact_large_box_one_step(large_box_one_step):
    """128^3 box, 5% chains (6,291,456 beads): one FP64 step equals the oracle's bit for bit."""
    world0, ow = large_box_one_step
    world = world0.copy()
    eng = E.GB300DPDEngine("fp64")
    eng.Attach(world)
    eng.Run(1)
    assert np.array_equal(world.f, ow.f)
    assert np.array_equal(world.x, ow.x)
    assert np.array_equal(world.v, ow.v)


@pytest.mark.parametrize("force_kernel", [8, 9])
def test_fp32_large_box_one_step_force_error(large_box_one_step, force_kernel):
    """The HBM-roofline configuration itself (128^3, 6,291,456 beads from uniform random
    positions): one FP32 step against the oracle's FP64 step, |f_i - f_ref_i| <= 1e-5
    rms|f_ref| for every bead but the few with a pair closer than 0.01 (on this machine: chain
    beads i and i + 2 folded back onto each other, r ~ 0.004), whose force the FP32 storage of
    positions (2^-25 per offset) moves by ~1e-3; those are held to the propagated storage
    error, at most 10x the tolerance, and must be rare (fp32_force_check).  Positions within
    1e-6."""
    world0, ow = large_box_one_step
    world = world0.copy()
    eng = E.GB300DPDEngine("fp32")
    eng.SetConfigEntry("force_kernel", force_kernel)
    eng.Attach(world)
    eng.Run(1)
    err, n_close = fp32_force_check(world0, ow.x, ow.v, world.f, ow.f, FP32_FORCE_TOL)
    print(f"128^3 one-step FP32 force error {err:.3e} of rms|f|; {n_close} beads above 1e-5 "
          f"(close pairs)")
    assert np.max(np.abs(periodic_dx(world.x, ow.x, world.box))) < 1e-6


# ---------------------------------------------------------------------------- FP32

@pytest.mark.parametrize("force_kernel", [1, 6, 8, 9])
@pytest.mark.parametrize("name", [n for n in world_fixture_names() if n != "empty_world"])
def test_fp32_vs_reference(name, force_kernel):
    world, ref = load_world_fixture(name)
    eng = E.GB300DPDEngine("fp32")
    eng.SetConfigEntry("force_kernel", force_kernel)
    eng.Attach(world)
    eng.Run(1)
    assert world.t == ref["t"][0]
    err = force_rel_err(world.f, ref["f"][0])
    assert err <= FP32_FORCE_TOL, f"{name}: 1-step force error {err:.3e}"
    dx = periodic_dx(world.x, ref["x"][0], world.box)
    assert np.max(np.abs(dx)) < 1e-6


@pytest.mark.parametrize("force_kernel", [1, 6, 8, 9])
def test_fp32_polymer_box_one_and_ten_steps(force_kernel):
    world = W.make_polymer_box(32, chain_fraction=0.1, seed=2)
    ow = O.OracleWorld(world)
    eng = E.GB300DPDEngine("fp32")
    eng.SetConfigEntry("force_kernel", force_kernel)
    eng.Attach(world)
    eng.Run(1)
    ow.run(1, nthreads=16)
    err = force_rel_err(world.f, ow.f)
    assert err <= FP32_FORCE_TOL, f"1-step force error {err:.3e}"
    eng.Run(9)
    ow.run(9, nthreads=16)
    dx = np.max(np.abs(periodic_dx(world.x, ow.x, world.box)))
    dv = np.max(np.abs(world.v - ow.v))
    assert dx < FP32_X10_TOL, dx
    assert dv < FP32_V10_TOL, dv


def test_cell_assignment_bit_exact_on_attach():
    """The FP32 engine stores integer cells: floor of the downloaded position is the cell the
    GPU assigned; it must equal the reference's floor(x) for every bead."""
    world = W.make_polymer_box(24, chain_fraction=0.1, seed=5)
    ref_cells = O.OracleWorld(world).cell_index()
    for prec in ("fp32", "fp64"):
        eng = E.GB300DPDEngine(prec)
        w = world.copy()
        eng.Attach(w)
        x, _, _, _ = eng.read_state(0)
        fl = np.floor(x).astype(np.int64)
        L = w.box.astype(np.int64)
        cells = fl[:, 0] * L[1] * L[2] + fl[:, 1] * L[2] + fl[:, 2]
        assert np.array_equal(cells, ref_cells), prec


def test_fp32_cell_assignment_after_one_step():
    world = W.make_polymer_box(24, chain_fraction=0.1, seed=6)
    ow = O.OracleWorld(world)
    ow.run(1)
    eng = E.GB300DPDEngine("fp32")
    w = world.copy()
    eng.Attach(w)
    eng.Run(1)
    ref = np.floor(ow.x)
    got = np.floor(w.x)
    frac = ow.x - ref
    near_face = np.any((frac < 1e-6) | (frac > 1 - 1e-6), axis=1)
    mismatch = np.any(ref != got, axis=1)
    assert not np.any(mismatch & ~near_face)


# ---------------------------------------------------------------------------- determinism / batching

@pytest.mark.parametrize("prec", ["fp32", "fp64"])
def test_deterministic_run_to_run(prec):
    world = W.make_polymer_box(16, chain_fraction=0.1, seed=8)
    outs = []
    for _ in range(2):
        w = world.copy()
        eng = E.GB300DPDEngine(prec)
        eng.Attach(w)
        eng.Run(25)
        outs.append((w.x, w.v, w.f))
    for a, b in zip(*outs):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("prec", ["fp32", "fp64"])
def test_batch_equals_alone(prec):
    """Each world's result is identical whether it runs alone or in a batch."""
    worlds = [W.make_polymer_box(L, chain_fraction=0.05, seed=i + 1, a_wt=aw, gamma=g,
                                 gen_seed=100 + i)
              for i, (L, aw, g) in enumerate([(8, 30.0, 3.5), (13, 80.0, 5.5), (10, 55.0, 4.0)])]
    alone = []
    for w in worlds:
        ww = w.copy()
        eng = E.GB300DPDEngine(prec)
        eng.Attach(ww)
        eng.Run(20)
        alone.append(ww)
    batch = [w.copy() for w in worlds]
    eng = E.GB300DPDEngine(prec)
    eng.AttachBatch(batch)
    eng.Run(20)  # reads every world back with pdpd_read_states
    for i, (a, b) in enumerate(zip(alone, batch)):
        assert a.t == b.t
        assert np.array_equal(a.x, b.x)
        assert np.array_equal(a.v, b.v)
        assert np.array_equal(a.f, b.f)
        x, v, f, t = eng.read_state(i)  # the per-world read gives the same state
        assert t == b.t and np.array_equal(x, b.x) and np.array_equal(v, b.v) and np.array_equal(f, b.f)
    # pdpd_read_states wants one view per attached world
    views = (E.PdpdStateView * 2)()
    assert E.lib().pdpd_read_states(eng._h, 2, views, 24) == 1  # PDPD_E_INVALID
    assert "views for a batch of 3 worlds" in E.lib().pdpd_last_error(eng._h).decode()


@pytest.mark.parametrize("prec", ["fp32", "fp64"])
def test_batch_with_an_empty_world(prec):
    """A world without beads in a batch: the others step as alone, and the batch read-back
    (pdpd_read_states) returns it empty."""
    empty, _ = load_world_fixture("empty_world")
    a = W.make_polymer_box(9, chain_fraction=0.1, seed=21)
    b = W.make_water(7, seed=22)
    alone = []
    for w in (a, b):
        ww = w.copy()
        eng = E.GB300DPDEngine(prec)
        eng.Attach(ww)
        eng.Run(12)
        alone.append(ww)
    batch = [a.copy(), empty.copy(), b.copy()]
    eng = E.GB300DPDEngine(prec)
    eng.AttachBatch(batch)
    eng.Run(12)
    assert batch[1].x.shape == (0, 3) and batch[1].t == empty.t + 12
    for w_alone, w_batch in zip(alone, (batch[0], batch[2])):
        assert np.array_equal(w_alone.x, w_batch.x) and np.array_equal(w_alone.v, w_batch.v)
        assert np.array_equal(w_alone.f, w_batch.f) and w_alone.t == w_batch.t


LAUNCH_CONFIGS = {
    # Every full-shell FP32 force kernel (shared-memory brick, any brick shape; thread per bead
    # from global memory) adds the same pair terms in the same order with the same roundings,
    # so all of them give bit-identical trajectories.
    "fp32": ({}, {"use_graphs": 0}, {"grid_blocks": 3}, {"graph_steps": 5},
             {"force_kernel": 1}, {"force_kernel": 1, "list_capacity": 1},
             {"list_capacity": 1}, {"list_capacity": 3, "force_kernel": 6},
             {"brick_x": 2, "brick_y": 2, "brick_z": 2}, {"brick_x": 8, "brick_y": 4, "brick_z": 8},
             {"force_kernel": 6}, {"force_kernel": 6, "list_capacity": 2},
             {"force_kernel": 6, "brick_x": 3, "brick_y": 5, "brick_z": 7},
             {"force_kernel": 8}, {"force_kernel": 8, "brick_x": 4, "brick_y": 8, "brick_z": 8},
             {"force_kernel": 8, "list_capacity": 3, "brick_x": 3, "brick_y": 5, "brick_z": 7}),
    # The half-shell kernel sums each bead's pair forces in fixed point (integer sums: any
    # order), so its trajectory is the same whatever its brick shape, grid or graph use.
    "fp32_half": ({"force_kernel": 9}, {"force_kernel": 9, "grid_blocks": 3},
                  {"force_kernel": 9, "use_graphs": 0}, {"force_kernel": 9, "graph_steps": 5},
                  {"force_kernel": 9, "brick_x": 4, "brick_y": 8, "brick_z": 8},
                  {"force_kernel": 9, "brick_x": 3, "brick_y": 5, "brick_z": 7},
                  {"force_kernel": 9, "brick_x": 1, "brick_y": 1, "brick_z": 1},
                  {"force_kernel": 9, "brick_y": 1, "brick_x": 12, "brick_z": 12},
                  {"force_kernel": 9, "brick_x": 2, "brick_y": 2, "brick_z": 12}),
    "fp64": ({}, {"use_graphs": 0}, {"list_capacity": 1}, {"list_capacity": 5, "grid_blocks": 3},
             {"graph_steps": 5}),
}


def test_autotune_and_mid_run_reconfiguration_keep_the_trajectory():
    """The autotuner times kernel variants and brick shapes on the run's own steps, and the
    kernel / brick shape can change between runs: none of it changes the FP32 trajectory."""
    world = W.make_polymer_box(16, chain_fraction=0.1, seed=12)
    ref = world.copy()
    e1 = E.GB300DPDEngine("fp32")
    e1.Attach(ref)
    e1.Run(80)
    w = world.copy()
    e2 = E.GB300DPDEngine("fp32")
    e2.SetConfigEntry("autotune", 1)
    e2.Attach(w)
    e2.Run(65)  # the autotuner's warm-up and trials take the first 49 steps
    cfg = {n: v for n, _, v in e2.GetConfigEntries()}
    assert "trials" in cfg["autotune"]
    e2.SetConfigEntry("force_kernel", 6 if cfg["force_kernel"] != "6" else 8)
    e2.SetConfigEntry("brick_z", 8)
    e2.Run(15)
    assert w.t == ref.t == 80
    assert np.array_equal(w.x, ref.x) and np.array_equal(w.v, ref.v) and np.array_equal(w.f, ref.f)


def clustered_world():
    """8^3 box with half the beads packed into a 2x2x2-cell corner: the halo of a brick there
    holds far more beads than the shared-memory budget, so the brick kernel falls back to the
    global-memory gather for it."""
    w = W.make_water(8, seed=5, dt=0.005)
    rng = np.random.default_rng(7)
    half = w.n_beads // 2
    w.x[:half] = 3.0 + 2.0 * rng.random((half, 3))
    return w


@pytest.mark.parametrize("force_kernel", [6, 8])
def test_fp32_brick_overflow_fallback(force_kernel):
    world = clustered_world()
    ref = world.copy()
    e1 = E.GB300DPDEngine("fp32")
    e1.SetConfigEntry("force_kernel", 1)
    e1.Attach(ref)
    e1.Run(2)
    w = world.copy()
    e2 = E.GB300DPDEngine("fp32")
    e2.SetConfigEntry("force_kernel", force_kernel)
    e2.Attach(w)
    e2.Run(2)
    assert np.array_equal(w.x, ref.x) and np.array_equal(w.f, ref.f)
    ow = O.OracleWorld(world)
    ow.run(1)
    w1 = world.copy()
    e3 = E.GB300DPDEngine("fp32")
    e3.SetConfigEntry("force_kernel", force_kernel)
    e3.Attach(w1)
    e3.Run(1)
    assert force_rel_err(w1.f, ow.f) <= FP32_FORCE_TOL


@pytest.mark.parametrize("variant", sorted(LAUNCH_CONFIGS))
def test_launch_configurations_agree(variant):
    prec = variant.split("_")[0]
    world = W.make_polymer_box(12, chain_fraction=0.1, seed=9)
    results = []
    for cfg in LAUNCH_CONFIGS[variant]:
        w = world.copy()
        eng = E.GB300DPDEngine(prec)
        for k, v in cfg.items():
            eng.SetConfigEntry(k, v)
        eng.Attach(w)
        eng.Run(17)
        results.append((w.x, w.v, w.f))
    for r in results[1:]:
        for a, b in zip(results[0], r):
            assert np.array_equal(a, b)


# ---------------------------------------------------------------------------- interval runs

@pytest.mark.parametrize("prec", ["fp32", "fp64"])
def test_run_intervals_matches_plain_run_and_rolls_back(prec):
    world = W.make_polymer_box(10, chain_fraction=0.1, seed=4)
    plain = world.copy()
    e1 = E.GB300DPDEngine(prec)
    e1.Attach(plain)
    e1.Run(30)

    w = world.copy()
    e2 = E.GB300DPDEngine(prec)
    e2.Attach(w)
    seen = []

    def cb():
        seen.append(w.t)
        return len(seen) < 3

    done = e2.Run(-1, 10, cb)
    assert done == 30
    assert seen == [10, 20, 30]
    assert w.t == 30
    assert np.array_equal(w.x, plain.x)
    assert np.array_equal(w.v, plain.v)
    assert np.array_equal(w.f, plain.f)
    # the engine stopped at the reported interval: continuing equals an uninterrupted run
    e2.Run(7)
    e1.Run(7)
    assert np.array_equal(w.x, plain.x)
    assert np.array_equal(w.f, plain.f)


def test_run_intervals_count():
    world = W.make_water(6, seed=3)
    eng = E.GB300DPDEngine("fp32")
    eng.Attach(world)
    calls = []
    done = eng.Run(4, 5, lambda: calls.append(world.t) or True)
    assert done == 20 and calls == [5, 10, 15, 20]
    assert eng.Run(0, 5, lambda: True) == 0


# ---------------------------------------------------------------------------- errors

@pytest.mark.parametrize("prec", ["fp32", "fp64"])
def test_snapped_bond_raises(prec):
    b = W.WorldBuilder((6, 6, 6), 1, [[25.0]], [[4.5]], dt=0.01)
    b.add_polymer_type([0, 0], [(0, 1, 128.0, 0.5)])
    b.add_polymer(0, [(1.0, 1.0, 1.0), (3.5, 1.0, 1.0)])
    eng = E.GB300DPDEngine(prec)
    eng.Attach(b.build())
    with pytest.raises(RuntimeError, match="snapped"):
        eng.Run(1)


def test_out_of_box_rejected_on_attach():
    w = W.make_water(4)
    w.x[3, 1] = 4.0
    eng = E.GB300DPDEngine("fp32")
    with pytest.raises(RuntimeError, match="outside the box"):
        eng.Attach(w)


def test_run_before_attach_is_an_error():
    eng = E.GB300DPDEngine("fp32")
    with pytest.raises(RuntimeError, match="PDPD_E_STATE"):
        eng.Run(1)


# ---------------------------------------------------------------------------- full-size properties

def test_full_size_momentum_and_determinism():
    """128^3 (6.3M beads) FP32: total momentum stays ~0 (pair forces are equal and opposite up
    to FP32 rounding) and two runs are bit-identical."""
    world = W.make_polymer_box(128, chain_fraction=0.05, seed=3)
    res = []
    for _ in range(2):
        w = world.copy()
        eng = E.GB300DPDEngine("fp32")
        eng.Attach(w)
        eng.Run(20)
        res.append(w)
    assert np.array_equal(res[0].x, res[1].x)
    p = res[0].v.sum(axis=0)
    assert np.max(np.abs(p)) / res[0].n_beads < 1e-5
    assert res[0].t == 20


# ---------------------------------------------------------------------------- reference test suite

@pytest.mark.parametrize("prec,force_kernel", [("fp64", None), ("fp32", None), ("fp32", 9)])
def test_reference_testbase_suite_replay(prec, force_kernel):
    """The reference's own 225-case engine test suite (TestBase families of test_engine.cpp),
    replayed segment by segment from the reference engine's recorded input states: the FP64
    engine reproduces every output bit for bit (so every property the suite checks on the
    reference engine holds for it); the FP32 engine -- its default kernels, and the half-shell
    kernel -- stays within the FP32 tolerances on the short segments and finishes every
    segment."""
    from _helpers import load_testbase, world_at
    cases = load_testbase()
    eng = E.GB300DPDEngine(prec)
    if force_kernel:
        eng.SetConfigEntry("force_kernel", force_kernel)
    checked = 0
    for name, world, segs in cases:
        for todo, t_in, s_in, t_out, s_out in segs:
            w = world_at(world, t_in, s_in)
            eng.Attach(w)
            eng.Run(todo)
            assert w.t == t_out, name
            got = np.hstack([w.x, w.v, w.f])
            if prec == "fp64":
                assert np.array_equal(got, s_out), f"{name}: segment t={t_in}+{todo}"
            else:
                assert np.all(np.isfinite(got)), name
                if todo == 1 and w.n_beads > 1:
                    assert force_rel_err(w.f, s_out[:, 6:9]) <= FP32_FORCE_TOL, name
            checked += 1
    assert checked == 900
