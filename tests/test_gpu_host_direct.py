"""Direct host copies (config ``host_direct``): the attach's upload and the read-backs done by a
kernel that reads and writes the caller's host arrays itself, where the device reaches pageable
host memory through the host's page tables (Grace-Blackwell over NVLink-C2C), against the staged
copies (pinned buffers and DMA, ``host_direct`` 0).

Both must give the same state to the bit, packed and strided (the C++ adapter's 88-byte bead
records), over segments of several copy chunks and odd lengths, with fields left out of a
read-back untouched, and with the callers' arrays untouched when a world has failed.
"""

import ctypes as C

import numpy as np
import pytest

import pdpd_engine as E
import pdpd_world as W
from test_gpu_boundary import BEAD, attach_strided, bead_records, non_vector_bytes

pytestmark = pytest.mark.gpu


def _engine(precision, direct):
    eng = E.GB300DPDEngine(precision)
    eng.SetConfigEntry("host_direct", direct)
    return eng


def _batch():
    # 16^3 polymer box: 12,288 beads = 36,864 words per vector array (three copy chunks, the
    # last partial); a 5x7x3 water box of 315 beads (odd word counts); a 2^3 box of 24
    return [W.make_polymer_box(16, chain_fraction=0.1, seed=41), W.make_water((5, 7, 3), seed=42),
            W.make_water(2, seed=43)]


def test_device_reports_pageable_host_access():
    """Which path the default takes on this device (informational: the staged path is correct
    everywhere, the direct one only where the device reaches pageable host memory)."""
    eng = E.GB300DPDEngine("fp32")
    eng.SetConfigEntry("host_direct", 1)  # (the default, whatever the test run forces)
    cfg = {n: v for n, _, v in eng.GetConfigEntries()}
    if "staged" in cfg["host_direct"]:
        pytest.skip("host_direct: " + cfg["host_direct"])
    assert cfg["host_direct"] == "1"


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_batch_direct_equals_staged(precision):
    out = {}
    for direct in (0, 1):
        ws = [w.copy() for w in _batch()]
        eng = _engine(precision, direct)
        eng.AttachBatch(ws)
        eng.Run(9)  # reads every world back into ws
        out[direct] = ws
    for a, b in zip(out[0], out[1]):
        assert a.t == b.t
        assert np.array_equal(a.x, b.x) and np.array_equal(a.v, b.v) and np.array_equal(a.f, b.f)


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_strided_records_direct_equals_staged(precision):
    world = W.make_polymer_box(12, chain_fraction=0.1, seed=44)
    res = {}
    for direct in (0, 1):
        rec = bead_records(world)
        marks = non_vector_bytes(rec)
        eng = _engine(precision, direct)
        attach_strided(eng, world, rec)
        eng._check(E.lib().pdpd_run(eng._h, 6), "Run")
        base = rec.ctypes.data
        t = C.c_int64(0)
        eng._check(E.lib().pdpd_read_state(eng._h, 0, base + 16, base + 40, base + 64, BEAD.itemsize,
                                           C.byref(t)), "read_state")
        assert np.array_equal(non_vector_bytes(rec), marks), "bytes outside x/v/f were written"
        res[direct] = (t.value, rec.copy())
    assert res[0][0] == res[1][0]
    for k in ("x", "v", "f"):
        assert np.array_equal(res[0][1][k], res[1][1][k])


def test_read_state_leaves_fields_not_asked_for():
    world = W.make_polymer_box(10, chain_fraction=0.1, seed=45)
    got = {}
    for direct in (0, 1):
        eng = _engine("fp32", direct)
        eng.Attach(world.copy())
        eng._check(E.lib().pdpd_run(eng._h, 4), "Run")
        x = np.zeros((world.n_beads, 3))
        f = np.zeros((world.n_beads, 3))
        v = np.full((world.n_beads, 3), 7.0)
        eng._check(E.lib().pdpd_read_state(eng._h, 0, x.ctypes.data, None, f.ctypes.data, 24, None),
                   "read_state")
        assert np.all(v == 7.0)
        got[direct] = (x, f)
    assert np.array_equal(got[0][0], got[1][0]) and np.array_equal(got[0][1], got[1][1])


@pytest.mark.parametrize("direct", [0, 1])
def test_failed_world_leaves_arrays_untouched(direct):
    b = W.WorldBuilder((6, 6, 6), 1, [[25.0]], [[4.5]], dt=0.01)
    b.add_polymer_type([0, 0], [(0, 1, 128.0, 0.5)])
    b.add_polymer(0, [(1.0, 1.0, 1.0), (3.5, 1.0, 1.0)])
    w = b.build()
    eng = _engine("fp64", direct)
    eng.Attach(w)
    with pytest.raises(RuntimeError, match="snapped"):
        eng.Run(1)
    dst = w.copy()
    x0 = dst.x.copy()
    with pytest.raises(RuntimeError, match="snapped"):
        eng.read_states(into=[dst])
    assert np.array_equal(dst.x, x0)


@pytest.mark.parametrize("direct", [0, 1])
def test_out_of_box_on_attach_either_path(direct):
    w = W.make_water(4)
    w.x[3, 1] = 4.0
    with pytest.raises(RuntimeError, match="outside the box"):
        _engine("fp32", direct).Attach(w)


def test_read_back_into_fresh_arrays():
    """Arrays the process has never written (np.empty: pages not yet mapped) as read-back
    destinations: the host touches their pages before the copy kernel writes them."""
    world = W.make_polymer_box(24, chain_fraction=0.05, seed=46)  # 41,472 beads, ~1 MB per vector array
    got = {}
    for direct in (0, 1):
        eng = _engine("fp32", direct)
        eng.Attach(world.copy())
        eng._check(E.lib().pdpd_run(eng._h, 3), "Run")
        x, v, f = (np.empty((world.n_beads, 3)) for _ in range(3))
        t = C.c_int64(0)
        eng._check(E.lib().pdpd_read_state(eng._h, 0, x.ctypes.data, v.ctypes.data, f.ctypes.data, 24,
                                           C.byref(t)), "read_state")
        got[direct] = (t.value, x, v, f)
    assert got[0][0] == got[1][0]
    for a, b in zip(got[0][1:], got[1][1:]):
        assert np.array_equal(a, b)


def _ragged_world(n, seed, offset_arrays=False):
    """A water-like world of exactly n beads (n from 1 up), optionally with x, v, f held 8 bytes
    into a larger buffer (8-byte but not 16-byte aligned arrays)."""
    rng = np.random.default_rng(seed)
    L = np.array([6, 5, 7], np.int32)
    x = rng.random((n, 3)) * L[None, :]
    v = rng.standard_normal((n, 3))
    w = W._assemble_monomer_world(L, x, v, np.array([[25.0]]), np.array([[4.5]]), 0.02, seed, 0, 1)
    if offset_arrays:
        for k in ("x", "v", "f"):
            buf = np.empty(3 * n + 1)
            a = buf[1:].reshape(n, 3)
            a[:] = getattr(w, k)
            setattr(w, k, a)
    return w


RAGGED = [1, 5, 7, 24, 127, 128, 129, 133, 134, 255, 262, 1000]


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_ragged_worlds_and_misaligned_arrays_direct_equals_staged(precision):
    """Worlds of 1 to 1000 beads (tile tails and the lines a tile shares with the next), some
    with arrays 8 bytes off a 16-byte boundary: the read-back kernel writes whole 128-byte
    lines, so these are its edge cases.  Every world read back at once and one at a time."""
    def make():
        return [_ragged_world(n, 100 + i, offset_arrays=bool(i % 2)) for i, n in enumerate(RAGGED)]
    out = {}
    for direct in (0, 1):
        ws = make()
        eng = _engine(precision, direct)
        eng.AttachBatch(ws)
        eng.Run(3)  # every world read back into its own arrays
        singles = [eng.read_state(i) for i in (0, 5, 7, len(RAGGED) - 1)]
        out[direct] = (ws, singles)
    (ws0, s0), (ws1, s1) = out[0], out[1]
    for a, b in zip(ws0, ws1):
        assert a.t == b.t
        assert np.array_equal(a.x, b.x) and np.array_equal(a.v, b.v) and np.array_equal(a.f, b.f)
    for (i, (a, b)) in zip((0, 5, 7, len(RAGGED) - 1), zip(s0, s1)):
        assert a[3] == b[3] == ws1[i].t
        for q in range(3):
            assert np.array_equal(a[q], b[q])
            assert np.array_equal(b[q], (ws1[i].x, ws1[i].v, ws1[i].f)[q])
