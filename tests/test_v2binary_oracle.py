"""The oracle's restatement of the v2binary state section (oracle/v2binary.py) against the
reference's own writer and reader (fixtures tests/golden/v2_*.npz, made by
oracle/ref/ref_harness), and the CVec3Half properties the reference's own test checks
(src/test/test_cvec3_half.cpp)."""

import numpy as np
import pytest

import v2binary as V
from _helpers import load_v2_fixture, v2_fixture_names


@pytest.mark.parametrize("name", v2_fixture_names())
def test_encode_equals_reference_writer(name):
    world, v2, _, _, _ = load_v2_fixture(name)
    _, section = V.split_file(v2)
    assert V.encode_section(world) == section


@pytest.mark.parametrize("name", v2_fixture_names())
def test_decode_equals_reference_reader(name):
    world, v2, x, v, f = load_v2_fixture(name)
    _, section = V.split_file(v2)
    dx, dv, df = V.decode_section(world, section)
    assert np.array_equal(dx, x) and np.array_equal(dv, v) and np.array_equal(df, f)
    # encode(decode(section)) == section: the decoded state is a fixed point of the codec
    assert V.encode_section(world, dx, dv, df) == section


def test_cvec3half_integers_are_exact():
    xs = np.arange(-255, 256, dtype=np.float64)
    vec = np.stack(np.meshgrid(xs, xs[::7], xs[::13], indexing="ij"), axis=-1).reshape(-1, 3)
    assert np.array_equal(V.cvec3half_decode(V.cvec3half_encode(vec)), vec)


def test_cvec3half_relative_error():
    rng = np.random.default_rng(4)
    vec = rng.standard_normal((100000, 3)) * np.exp(rng.uniform(-9, 8, (100000, 1)))
    got = V.cvec3half_decode(V.cvec3half_encode(vec))
    largest = np.max(np.abs(vec), axis=1)
    live = largest >= 2.0 ** -15  # frexp exponent >= -14
    assert np.all(np.abs(got - vec)[live] / largest[live, None] < 1.0 / 128)
    tr, gr = np.linalg.norm(vec[live], axis=1), np.linalg.norm(got[live], axis=1)
    assert np.all(np.abs(tr - gr) / gr < 1.0 / 64)
    assert not got[~live].any()


def test_cvec3half_rejects_non_finite_and_overflow():
    for bad in ([np.nan, 0, 0], [0, np.inf, 0], [40000.0, 0, 0], [32767.9, 0, 0]):
        with pytest.raises(V.V2Error):
            V.cvec3half_encode(np.array([bad], float))
