"""The per-pair force log (pdpd_log_pair_terms), the counterpart of the reference's ForceLogging:
against the reference's own log of the same world (tests/golden/pair_log_polymer10.npz, made
by the reference's half-step engine with a logger installed; tests/golden/make_golden.py).

The FP64 engine's records equal the reference's bit for bit, pair for pair, in the same order
for each home bead; the logging step is an ordinary step (the state afterwards equals Run's).
The FP32 engine's records agree within FP32 precision."""

import os

import numpy as np
import pytest

import pdpd_engine as E
import pdpd_world as W

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "pair_log_polymer10.npz")
SCALARS = ["dr", "inv_root_dt", "gammap", "rng", "con", "diss", "rng_scale", "rand"]


def _golden():
    d = np.load(GOLDEN)
    world = W.read_pdw1(d["world"].tobytes())
    return world, d


def _by_home(t, home, other):
    """(t, home hash) -> the sequence of other hashes, in record order."""
    seq = {}
    for k in range(len(t)):
        seq.setdefault((int(t[k]), int(home[k])), []).append(k)
    return seq


def _log(prec, world, ids, steps):
    eng = E.GB300DPDEngine(prec)
    w = world.copy()
    eng.Attach(w)
    recs = [eng.log_pair_terms(ids) for _ in range(steps)]
    return eng, np.concatenate(recs)


def test_fp64_pair_log_equals_the_reference_log():
    world, g = _golden()
    ids, steps = g["ids"], int(g["steps"])
    eng, r = _log("fp64", world, ids, steps)
    assert len(r) == len(g["t"])
    hashes = world.hashes()
    assert set(r["home_hash"]) == set(hashes[ids])
    assert np.array_equal(r["home_hash"], hashes[r["home_id"]])
    assert np.array_equal(r["other_hash"], hashes[r["other_id"]])
    mine, ref = _by_home(r["t"], r["home_hash"], r["other_hash"]), _by_home(g["t"], g["home_hash"], g["other_hash"])
    assert mine.keys() == ref.keys()
    for key, ks in mine.items():
        kr = ref[key]
        # the same pairs in the same order (the reference's direction walk)
        assert np.array_equal(r["other_hash"][ks], g["other_hash"][kr]), key
        for name in SCALARS:
            assert np.array_equal(r[name][ks], g[name][kr]), (key, name)
        assert np.array_equal(r["dx"][ks], g["dx"][kr]), key
        assert np.array_equal(r["f"][ks], g["f"][kr]), key


def test_logging_steps_are_ordinary_steps():
    world, g = _golden()
    eng, _ = _log("fp64", world, g["ids"], 3)
    logged = world.copy()
    eng.read_state(0, into=logged)
    plain = world.copy()
    e2 = E.GB300DPDEngine("fp64")
    e2.Attach(plain)
    e2.Run(3)
    assert logged.t == plain.t == 3
    assert np.array_equal(logged.x, plain.x)
    assert np.array_equal(logged.v, plain.v)
    assert np.array_equal(logged.f, plain.f)


def test_fp32_pair_log_within_fp32_precision():
    world, g = _golden()
    _, r = _log("fp32", world, g["ids"], int(g["steps"]))
    assert len(r) == len(g["t"])  # no pair of this world is within FP32 rounding of r = 1
    mine, ref = _by_home(r["t"], r["home_hash"], r["other_hash"]), _by_home(g["t"], g["home_hash"], g["other_hash"])
    assert mine.keys() == ref.keys()
    fscale = np.sqrt(np.mean(np.sum(g["f"] ** 2, axis=1)))
    for key, ks in mine.items():
        # the FP32 cell lists hold a cell's lower-z-half beads first (then id order), so the
        # pairs of one direction may come in another order: match them by partner
        kr = [ref[key][i] for i in np.argsort(g["other_hash"][ref[key]], kind="stable")]
        ks = [ks[i] for i in np.argsort(r["other_hash"][ks], kind="stable")]
        assert np.array_equal(r["other_hash"][ks], g["other_hash"][kr]), key
        assert np.array_equal(r["rng"][ks], g["rng"][kr])  # the RNG is bit-exact in FP32 too
        assert np.allclose(r["dr"][ks], g["dr"][kr], rtol=0, atol=1e-6)
        assert np.allclose(r["dx"][ks], g["dx"][kr], rtol=0, atol=1e-6)
        for name in ("con", "diss", "rand", "rng_scale", "gammap"):
            assert np.allclose(r[name][ks], g[name][kr], rtol=1e-5, atol=1e-6 * fscale), (key, name)
        assert np.max(np.abs(r["f"][ks] - g["f"][kr])) <= 1e-5 * fscale, key


def test_pair_log_rejects_bad_ids():
    world, g = _golden()
    eng = E.GB300DPDEngine("fp64")
    eng.Attach(world.copy())
    with pytest.raises(RuntimeError, match="out of range"):
        eng.log_pair_terms([world.n_beads])
    # duplicates are one bead, and no bead gives no records (the step still runs)
    a = eng.log_pair_terms([5, 5])
    assert len(a) > 0 and set(a["home_id"]) == {5}
    assert len(eng.log_pair_terms([])) == 0


def test_force_log_lines_use_the_reference_format():
    world, g = _golden()
    _, r = _log("fp64", world, g["ids"][:1], 1)
    lines = E.force_log_lines(r[:1])
    assert len(lines) == 10
    h0 = int(r["home_hash"][0]) & 0x0FFFFFFF
    assert lines[0].startswith(f"Prop,0,{h0},")
    assert [ln.split(",")[5] for ln in lines] == [n for n, _ in E.PAIR_LOG_PROPERTIES]
    assert all(len(ln.split(",")) == 9 for ln in lines)
