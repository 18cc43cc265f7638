"""The reference's per-pair force log fixture (tests/golden/pair_log_polymer10.npz, written by
the reference's half-step engine through a ForceLogging logger) is self-consistent, and the
text rendering of pair records follows the reference's FileLogger format.  CPU only."""

import os

import numpy as np

import pdpd_engine as E
import pdpd_world as W

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "pair_log_polymer10.npz")


def test_reference_pair_log_is_consistent():
    d = np.load(GOLDEN)
    world = W.read_pdw1(d["world"].tobytes())
    hashes = world.hashes()
    assert set(np.unique(d["home_hash"])) == set(hashes[d["ids"]])
    assert set(np.unique(d["t"])) == set(range(int(d["steps"])))
    # calc_force's relations among the logged terms (dpd_maths_core_half_step.hpp:98-153)
    dr = d["dr"]
    assert np.all((dr > 0) & (dr < 1))
    assert np.allclose(np.linalg.norm(d["dx"], axis=1), dr, rtol=1e-12)
    assert np.allclose(d["inv_root_dt"], np.sqrt(24.0 / world.dt), rtol=1e-15)
    assert np.all((d["rng"] >= -0.5) & (d["rng"] < 0.5))
    assert np.allclose(d["rand"], d["rng_scale"] * d["rng"], rtol=1e-15, atol=0)
    assert np.allclose(d["rng_scale"] ** 2, d["gammap"] * 24.0 / world.dt, rtol=1e-12)
    e = d["dx"] / dr[:, None]
    assert np.allclose(d["f"], e * (d["con"] + d["diss"] + d["rand"])[:, None], rtol=1e-12, atol=1e-12)


def test_force_log_lines_format():
    r = np.zeros(2, E.PAIR_TERMS_DTYPE)
    r["t"] = 7
    r["home_hash"] = [0x1000002A, 0x00000003]
    r["other_hash"] = [0x20000005, 0x1000002A]
    r["dx"] = [[0.25, -0.5, 0.125], [1e-7, 2.5, 3]]
    r["dr"] = [0.5, 0.75]
    r["rng"] = [-0.5, 0.25]
    lines = E.force_log_lines(r, prefix="A")
    assert len(lines) == 20
    assert lines[0] == "AProp,7,42,5,,dx,0.25,-0.5,0.125"
    assert lines[1] == "AProp,7,42,5,,dr,0.5,,"
    assert lines[4] == "AProp,7,42,5,,dpd-rng,-0.5,,"   # negative: printed as a double
    assert lines[10] == "AProp,7,3,42,,dx,1e-07,2.5,3"  # 3.0 is an integer in [0, 2^32)
    assert [ln.split(",")[5] for ln in lines[:10]] == [n for n, _ in E.PAIR_LOG_PROPERTIES]
