"""v2binary snapshots encoded and decoded on the GPU, against the reference's own writer and
reader (fixtures tests/golden/v2_*.npz) and the oracle's restatement (oracle/v2binary.py).
Integer/byte work: every comparison is exact."""

import numpy as np
import pytest

import pdpd_engine as E
import pdpd_world as W
import v2binary as V
from _helpers import load_v2_fixture, v2_fixture_names

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", v2_fixture_names())
def test_fp64_encode_equals_reference_writer(name):
    world, v2, _, _, _ = load_v2_fixture(name)
    _, section = V.split_file(v2)
    eng = E.GB300DPDEngine("fp64")
    eng.Attach(world.copy())
    assert eng.v2binary_prepare() == len(section)
    assert eng.v2binary_encode().tobytes() == section


@pytest.mark.parametrize("name", v2_fixture_names())
def test_decode_equals_reference_reader(name):
    world, v2, x, v, f = load_v2_fixture(name)
    _, section = V.split_file(v2)
    eng = E.GB300DPDEngine("fp64")
    w = world.copy()
    w.x = np.full_like(w.x, 0.5)  # the state comes from the section only
    w.v[:] = 0.0
    w.f[:] = 0.0
    eng.Attach(w)
    eng.v2binary_prepare()
    eng.v2binary_decode(section)
    assert np.array_equal(w.x, x) and np.array_equal(w.v, v) and np.array_equal(w.f, f)
    assert eng.v2binary_encode().tobytes() == section  # the decoded state re-encodes to the same bytes


@pytest.mark.parametrize("prec", ["fp32", "fp64"])
def test_encode_after_a_run_equals_oracle_codec(prec):
    world = W.make_polymer_box(12, chain_fraction=0.1, seed=6)
    eng = E.GB300DPDEngine(prec)
    w = world.copy()
    eng.Attach(w)
    eng.v2binary_prepare()
    eng.Run(25)  # w now holds the engine's x, v, f
    assert eng.v2binary_encode().tobytes() == V.encode_section(w)


def test_non_sequential_polymer_ids_and_batches():
    a = W.make_polymer_box(6, chain_fraction=0.3, seed=4)
    b = W.make_water(5, seed=2)
    eng = E.GB300DPDEngine("fp64")
    ws = [b.copy(), a.copy()]
    eng.AttachBatch(ws)
    pids = (np.arange(len(a.poly_type), dtype=np.uint32) * 3 + 7)
    eng.v2binary_prepare(1, polymer_ids=pids)
    eng.v2binary_prepare(0)
    assert eng.v2binary_encode(1).tobytes() == V.encode_section(a, polymer_ids=pids)
    assert eng.v2binary_encode(0).tobytes() == V.encode_section(b)


def test_round_trip_large_box():
    """64^3 box (786,432 beads) after 20 FP32 steps: decode(encode(state)) re-encodes to the
    same bytes, and the decoded state is within the format's resolution of the state."""
    world = W.make_polymer_box(64, chain_fraction=0.05, seed=9)
    eng = E.GB300DPDEngine("fp32")
    w = world.copy()
    eng.Attach(w)
    n = eng.v2binary_prepare()
    eng.Run(20)
    x0, v0, f0 = w.x.copy(), w.v.copy(), w.f.copy()
    sec = eng.v2binary_encode().tobytes()
    assert len(sec) == n
    eng.v2binary_decode(sec)
    assert eng.v2binary_encode().tobytes() == sec
    d = np.abs(w.x - x0)
    d = np.minimum(d, np.asarray(w.box, float) - d)
    assert d.max() <= 0.5 / 65536 + 1e-12
    for got, ref in ((w.v, v0), (w.f, f0)):
        big = np.max(np.abs(ref), axis=1)
        assert np.all(np.abs(got - ref).max(axis=1) <= big / 128 + 2.0 ** -15)
    eng.Run(5)  # the decoded state steps on


def test_errors():
    w = W.make_water(4, seed=3)
    w.f[5] = (1e5, 0.0, 0.0)
    eng = E.GB300DPDEngine("fp64")
    eng.Attach(w)
    with pytest.raises(RuntimeError, match="v2binary_prepare|not called"):
        eng.v2binary_encode()
    eng.v2binary_prepare()
    with pytest.raises(RuntimeError, match="CVec3Half"):
        eng.v2binary_encode()
    good = W.make_water(4, seed=3)
    eng2 = E.GB300DPDEngine("fp64")
    eng2.Attach(good)
    eng2.v2binary_prepare()
    sec = bytearray(eng2.v2binary_encode().tobytes())
    sec[0] ^= 1  # first polymer header: another polymer type
    with pytest.raises(RuntimeError, match="structure"):
        eng2.v2binary_decode(bytes(sec))
    with pytest.raises(RuntimeError, match="bytes"):
        eng2.v2binary_decode(bytes(sec[:-2]))
