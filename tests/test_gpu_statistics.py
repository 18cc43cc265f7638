"""Observables on the GPU (FP64 reductions) and the statistics of long FP32 runs against the
FP64 oracle.  Trajectories of a chaotic system separate after a few hundred steps; what must
agree is the thermodynamics: kinetic temperature, pressure, the per-type radial distribution
and the bond-length distribution, within statistical error -- an error measured from
independent runs, not assumed:

  * the 32^3 polymer box of the reference's 1000-step FP32-vs-FP64 configuration, in 8
    replicas (other seeds) run by the FP32 engine and by the oracle;
  * a 32-state slice of the 512-state grid, stepped together on one batched FP32 engine, the
    oracle running each state alone.

Each replica or state gives one difference GPU - oracle of its time-averaged observables; they
are independent, so the standard error of the mean difference is their spread / sqrt(count).
A difference passes when it is within 5 standard errors, and temperature and pressure also
within 0.5% and 1% of the oracle's (the engine's stated bounds for those two)."""

import numpy as np
import pytest

import oracle as O
import pdpd_engine as E
import pdpd_world as W

pytestmark = pytest.mark.gpu

SIGMAS = 5.0


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_gpu_observables_equal_oracle_on_the_same_state(prec):
    world = W.make_polymer_box(12, chain_fraction=0.1, seed=21)
    eng = E.GB300DPDEngine(prec)
    eng.Attach(world)
    eng.Run(5)  # world now holds the engine's x, v, f
    got = eng.observe(n_bins=40, n_bond_bins=50)
    ref = O.OracleWorld(world).observe(n_bins=40, n_bond_bins=50)
    assert got["ke2"] == pytest.approx(ref["ke2"], rel=1e-12)
    assert got["virial"] == pytest.approx(ref["virial"], rel=1e-12 if prec == "fp64" else 1e-6)
    assert np.allclose(got["momentum"], ref["momentum"], atol=1e-9)
    if prec == "fp64":  # same positions, same distance arithmetic: identical bins
        assert np.array_equal(got["rdf"], ref["rdf"])
        assert np.array_equal(got["bond_hist"], ref["bond_hist"])
    else:  # FP32 offsets move distances by ~1e-7: a pair on a bin edge may change bin
        assert np.abs(got["rdf"].astype(float) - ref["rdf"]).sum() <= 1e-4 * ref["rdf"].sum() + 2
        assert np.abs(got["bond_hist"].astype(float) - ref["bond_hist"]).sum() <= 2


# ---------------------------------------------------------------------------- helpers

def observe_series(samples, n, V):
    T = np.array([s["ke2"] / (3 * n) for s in samples])
    P = np.array([(s["ke2"] + s["virial"]) / (3 * V) for s in samples])
    rdf = np.array([s["rdf"].astype(float) for s in samples])
    bh = np.array([s["bond_hist"].astype(float) for s in samples])
    return T, P, rdf, bh


def assert_within(name, diff, se, floor=0.0):
    """|diff| <= SIGMAS * se elementwise, where se (and a small absolute floor for bins whose
    error estimate is zero) bound the error."""
    diff, se = np.asarray(diff, float), np.asarray(se, float)
    bound = SIGMAS * np.maximum(se, floor)
    bad = np.abs(diff) > bound
    assert not bad.any(), (name, np.argwhere(bad)[:5].tolist(), diff[bad][:5], bound[bad][:5])


def pooled_bin_se(d, c):
    """Standard error of the mean over axis 0 (replicas) of per-bin differences d, pooled over
    the bins: a bin's variance is taken as the larger of its own and k * c (c its mean count,
    k the median of var / c over the bins), since one bin's spread over a few replicas is
    itself too noisy to bound it."""
    var = d.var(axis=0, ddof=1)
    ok = c > 0
    k = np.median(var[ok] / c[ok]) if ok.any() else 0.0
    return np.sqrt(np.maximum(var, k * c) / d.shape[0])


def compare_states(worlds, gpu_samples, n_bins, n_bond_bins, equil, every, n_samples):
    """Run each world on the oracle (equil steps, then n_samples observations every `every`
    steps), and check the mean over the worlds of the GPU - oracle differences of the
    time-averaged T, P, mean bond length, RDF and bond histogram."""
    m = len(worlds)
    centers = (np.arange(n_bond_bins) + 0.5) * 2.0 / n_bond_bins
    dT, dP, dL, drdf, dbh, Tc, Pc, Lc, rdf_c, bh_c = ([] for _ in range(10))
    for i, w in enumerate(worlds):
        ow = O.OracleWorld(w)
        ow.run(equil, nthreads=16)
        c = [ow.observe(n_bins=n_bins, n_bond_bins=n_bond_bins, nthreads=16)]
        for _ in range(n_samples - 1):
            ow.run(every, nthreads=16)
            c.append(ow.observe(n_bins=n_bins, n_bond_bins=n_bond_bins, nthreads=16))
        n, V = w.n_beads, float(np.prod(w.box))
        Tg_, Pg_, rg_, bg_ = observe_series(gpu_samples[i], n, V)
        Tc_, Pc_, rc_, bc_ = observe_series(c, n, V)
        dT.append(Tg_.mean() - Tc_.mean())
        dP.append(Pg_.mean() - Pc_.mean())
        Tc.append(Tc_.mean())
        Pc.append(Pc_.mean())
        drdf.append(rg_.mean(0) - rc_.mean(0))
        rdf_c.append(rc_.mean(0))
        dbh.append(bg_.mean(0) - bc_.mean(0))
        bh_c.append(bc_.mean(0))
        if bc_.sum() > 0:
            lg_ = (bg_.sum(0) * centers).sum() / bg_.sum()
            lc_ = (bc_.sum(0) * centers).sum() / bc_.sum()
            dL.append(lg_ - lc_)
            Lc.append(lc_)
    dT, dP, dL, drdf, dbh = map(np.array, (dT, dP, dL, drdf, dbh))
    se = lambda d: d.std(axis=0, ddof=1) / np.sqrt(len(d))  # noqa: E731
    assert abs(dT.mean()) / np.mean(Tc) < 0.005, (dT.mean(), np.mean(Tc))
    assert abs(dP.mean()) / np.mean(Pc) < 0.01, (dP.mean(), np.mean(Pc))
    assert_within("T", dT.mean(), se(dT))
    assert_within("P", dP.mean(), se(dP))
    if len(dL) > 1:
        assert abs(dL.mean()) / np.mean(Lc) < 0.005, (dL.mean(), np.mean(Lc))
        assert_within("mean bond length", dL.mean(), se(dL))
    rc_mean = np.mean(rdf_c, axis=0)
    nt = rc_mean.shape[0]
    for ti in range(nt):
        for tj in range(ti, nt):
            ok = rc_mean[ti, tj] > 5  # bins with counts (r -> 0 is empty)
            if ok.any():
                assert_within(f"rdf[{ti},{tj}]", drdf.mean(0)[ti, tj][ok],
                              pooled_bin_se(drdf[:, ti, tj][:, ok], rc_mean[ti, tj][ok]), floor=0.5)
    bc_mean = np.mean(bh_c, axis=0)
    ok = bc_mean > 5
    if ok.any():
        assert_within("bond_hist", dbh.mean(0)[ok], pooled_bin_se(dbh[:, ok], bc_mean[ok]), floor=0.5)
    return dT.mean(), dP.mean()


def batched_gpu_samples(worlds, n_bins, n_bond_bins, equil, every, n_samples):
    """The worlds stepped together on one batched FP32 engine; per world, n_samples GPU
    observations (after equil steps, then every `every` steps)."""
    eng = E.GB300DPDEngine("fp32")
    eng.AttachBatch([w.copy() for w in worlds])
    eng.run_async(equil)
    eng.sync()
    g = [[] for _ in worlds]
    for k in range(n_samples):
        if k:
            eng.run_async(every)
            eng.sync()
        for i in range(len(worlds)):
            g[i].append(eng.observe(i, n_bins=n_bins, n_bond_bins=n_bond_bins))
    return g


# ---------------------------------------------------------------------------- the tests

def test_polymer_box_1000_steps_fp32_statistics_match_fp64_oracle():
    """The 32^3 polymer-solvent box (98,304 beads, 10% H-T5 chains) run 1000 steps by the
    FP32 engine and by the FP64 oracle, from the same start, in 8 replicas (seeds 2..9: other
    start positions, velocities and random streams).  The T beads (a_WT = a_HT = 75) keep
    aggregating over the whole run, so the observables drift and one run's time series has no
    stationary stretch long enough to measure its own error; replicas give the error instead:
    each replica's GPU - oracle difference of its time averages (steps 200..1000, every 40) is
    one independent sample.  (The replicas share one batched engine; a world's trajectory is
    the same alone and in a batch, bit for bit.)"""
    worlds = [W.make_polymer_box(32, chain_fraction=0.1, seed=2 + r) for r in range(8)]
    args = dict(n_bins=20, n_bond_bins=20, equil=200, every=40, n_samples=21)
    g = batched_gpu_samples(worlds, **args)
    dT, dP = compare_states(worlds, g, **args)
    print(f"32^3 polymer box, 8 replicas x 1000 steps: mean dT {dT:+.2e}, mean dP {dP:+.2e}")


def test_batched_grid_slice_fp32_statistics_match_fp64_oracle():
    """The first 32 states of the 512-state grid (sides 8..32, per-state a_WT and gamma, 5%
    chains) stepped 200 steps together on one batched FP32 engine, each state against the
    oracle run alone; time averages over steps 100..200 (every 10 steps)."""
    worlds = list(W.make_batched_grid(512, count=32))
    args = dict(n_bins=20, n_bond_bins=20, equil=100, every=10, n_samples=11)
    g = batched_gpu_samples(worlds, **args)
    dT, dP = compare_states(worlds, g, **args)
    print(f"512-state grid, first 32 states x 200 steps: mean dT {dT:+.2e}, mean dP {dP:+.2e}")
