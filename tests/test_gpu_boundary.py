"""The drop-in boundary's strided write-back, through the C ABI, as the C++ adapter uses it.

The adapter hands the engine `&state.beads[0].x[0]` with stride `sizeof(Bead)` and no copy
(reference include/dpd/core/dpd_state.hpp:141-158: bead_id, polymer_id, polymer_offset,
bead_type, polymer_type, is_monomer, then x, v, f as double[3]: 88 bytes, x at 16, v at 40,
f at 64).  The DPDEngine contract (dpd_engine.hpp:171-215) is that beads are not reordered
and that x, v, f are valid at the return of Run and at every interval callback.  These tests
drive pdpd_attach, pdpd_run, pdpd_read_state and pdpd_run_intervals (with an early stop)
with such records and require the vectors to equal a packed (stride 24) run bit for bit and
every other byte of the records to be left as it was.
"""

import ctypes as C

import numpy as np
import pytest

import pdpd_engine as E
import pdpd_world as W

pytestmark = pytest.mark.gpu

BEAD = np.dtype({"names": ["bead_id", "polymer_id", "polymer_offset", "bead_type", "polymer_type",
                           "is_monomer", "x", "v", "f"],
                 "formats": ["<u4", "<u4", "u1", "u1", "u1", "u1", ("<f8", 3), ("<f8", 3),
                             ("<f8", 3)],
                 "offsets": [0, 4, 8, 9, 10, 11, 16, 40, 64], "itemsize": 88})


def bead_records(world):
    rec = np.zeros(world.n_beads, BEAD)
    rec["bead_id"] = np.arange(world.n_beads)
    rec["polymer_id"] = world.polymer_id
    rec["polymer_offset"] = world.polymer_offset
    rec["bead_type"] = world.bead_type
    rec["polymer_type"] = world.polymer_type_of_bead
    rec["is_monomer"] = world.is_monomer
    rec["x"], rec["v"], rec["f"] = world.x, world.v, world.f
    return rec


def attach_strided(eng, world, rec):
    """pdpd_attach with x/v/f read from the 88-byte records."""
    fl = E._Flat(world)
    base = rec.ctypes.data
    fl.struct.x, fl.struct.v, fl.struct.f = base + 16, base + 40, base + 64
    fl.struct.bead_stride_bytes = BEAD.itemsize
    eng._check(E.lib().pdpd_attach(eng._h, C.byref(fl.struct)), "Attach")


def non_vector_bytes(rec):
    raw = rec.view(np.uint8).reshape(-1, BEAD.itemsize)
    return np.concatenate([raw[:, :16], raw[:, 88:]], axis=1).copy()


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_strided_attach_run_read_state(precision):
    world = W.make_polymer_box(8, chain_fraction=0.1, seed=4)
    rec = bead_records(world)
    rec["f"] = 0.0
    world.f[:] = 0.0
    marks = non_vector_bytes(rec)

    packed = world.copy()
    ep = E.GB300DPDEngine(precision)
    ep.Attach(packed)
    ep.Run(7)

    es = E.GB300DPDEngine(precision)
    attach_strided(es, world, rec)
    es._check(E.lib().pdpd_run(es._h, 7), "Run")
    t = C.c_int64(0)
    base = rec.ctypes.data
    es._check(E.lib().pdpd_read_state(es._h, 0, base + 16, base + 40, base + 64, BEAD.itemsize,
                                      C.byref(t)), "read_state")
    assert t.value == packed.t
    assert np.array_equal(rec["x"], packed.x)
    assert np.array_equal(rec["v"], packed.v)
    assert np.array_equal(rec["f"], packed.f)
    assert np.array_equal(non_vector_bytes(rec), marks), "bytes outside x/v/f were written"


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_strided_run_intervals_with_early_stop(precision):
    world = W.make_polymer_box(8, chain_fraction=0.1, seed=5)
    rec = bead_records(world)
    marks = non_vector_bytes(rec)

    # packed reference: the same intervals, stopped after the third callback
    packed = world.copy()
    ep = E.GB300DPDEngine(precision)
    ep.Attach(packed)
    seen_packed = []

    def cb_packed():
        seen_packed.append((packed.t, packed.x.copy(), packed.v.copy(), packed.f.copy()))
        return len(seen_packed) < 3

    done_packed = ep.Run(-1, 4, cb_packed)

    es = E.GB300DPDEngine(precision)
    attach_strided(es, world, rec)
    seen = []
    base = rec.ctypes.data

    def tramp(_user, t):
        seen.append((int(t), rec["x"].copy(), rec["v"].copy(), rec["f"].copy()))
        return 1 if len(seen) < 3 else 0

    fn = E.INTERVAL_FN(tramp)
    done = C.c_uint32(0)
    rc = E.lib().pdpd_run_intervals(es._h, -1, 4, base + 16, base + 40, base + 64, BEAD.itemsize,
                                    fn, None, C.byref(done))
    es._check(rc, "Run(intervals)")
    assert done.value == done_packed == 12
    assert len(seen) == len(seen_packed) == 3
    for (t, x, v, f), (tp, xp, vp, fp) in zip(seen, seen_packed):
        assert t == tp
        assert np.array_equal(x, xp) and np.array_equal(v, vp) and np.array_equal(f, fp)
    assert np.array_equal(non_vector_bytes(rec), marks), "bytes outside x/v/f were written"
    # after the early stop the device holds the reported state: one more step from it equals
    # one more step of the packed run
    es._check(E.lib().pdpd_run(es._h, 1), "Run")
    t = C.c_int64(0)
    es._check(E.lib().pdpd_read_state(es._h, 0, base + 16, base + 40, base + 64, BEAD.itemsize,
                                      C.byref(t)), "read_state")
    ep.Run(1)
    assert t.value == packed.t
    assert np.array_equal(rec["x"], packed.x) and np.array_equal(rec["v"], packed.v)
    assert np.array_equal(rec["f"], packed.f)
