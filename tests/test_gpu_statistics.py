"""Observables on the GPU (FP64 reductions) and the statistics of long FP32 runs against the
FP64 oracle.  Trajectories of a chaotic system separate after a few hundred steps; what must
agree is the thermodynamics: kinetic temperature, pressure, the per-type radial distribution
and the bond-length distribution, within statistical error."""

import numpy as np
import pytest

import oracle as O
import pdpd_engine as E
import pdpd_world as W

pytestmark = pytest.mark.gpu


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


def sample(run_step, observe, n_equil, n_samples, every):
    run_step(n_equil)
    out = []
    for _ in range(n_samples):
        run_step(every)
        out.append(observe())
    return out


def test_long_fp32_run_reproduces_fp64_oracle_statistics():
    """20^3 polymer box (24,000 beads, 10% H-T5 chains), 200 equilibration steps then 40
    samples 10 steps apart, FP32 GPU engine vs FP64 oracle from the same start."""
    world = W.make_polymer_box(20, chain_fraction=0.1, seed=31)
    n, V = world.n_beads, float(np.prod(world.box))
    n_bins, n_bond_bins = 25, 40

    eng = E.GB300DPDEngine("fp32")
    eng.Attach(world.copy())
    gpu = sample(lambda k: eng.run_async(k) or eng.sync(),
                 lambda: eng.observe(n_bins=n_bins, n_bond_bins=n_bond_bins), 200, 40, 10)
    ow = O.OracleWorld(world)
    cpu = sample(lambda k: ow.run(k, nthreads=16),
                 lambda: ow.observe(n_bins=n_bins, n_bond_bins=n_bond_bins, nthreads=16), 200, 40, 10)

    def summary(samples):
        T = np.array([s["ke2"] / (3 * n) for s in samples])
        P = np.array([(s["ke2"] + s["virial"]) / (3 * V) for s in samples])
        rdf = sum(s["rdf"].astype(float) for s in samples)
        bh = sum(s["bond_hist"].astype(float) for s in samples)
        return T, P, rdf, bh

    Tg, Pg, rdf_g, bh_g = summary(gpu)
    Tc, Pc, rdf_c, bh_c = summary(cpu)
    # temperature within 0.5% (the statistical error of each mean is ~0.1%)
    assert abs(Tg.mean() - Tc.mean()) / Tc.mean() < 0.005, (Tg.mean(), Tc.mean())
    # pressure within 1%
    assert abs(Pg.mean() - Pc.mean()) / Pc.mean() < 0.01, (Pg.mean(), Pc.mean())
    # RDF of every type pair with enough counts: bins agree within 5 Poisson sigmas (x3 for
    # the correlation of samples 10 steps apart)
    for ti in range(3):
        for tj in range(ti, 3):
            a, b = rdf_g[ti, tj], rdf_c[ti, tj]
            ok = (a + b) > 400
            z = np.abs(a - b)[ok] / np.sqrt(a + b)[ok]
            assert z.size == 0 or z.max() < 15, (ti, tj, z.max())
    # bond-length histogram: same mean bond length to 0.5%, bins within error
    centers = (np.arange(n_bond_bins) + 0.5) * 2.0 / n_bond_bins
    mg, mc = (bh_g * centers).sum() / bh_g.sum(), (bh_c * centers).sum() / bh_c.sum()
    assert abs(mg - mc) / mc < 0.005, (mg, mc)
    ok = (bh_g + bh_c) > 400
    z = np.abs(bh_g - bh_c)[ok] / np.sqrt(bh_g + bh_c)[ok]
    assert z.max() < 15, z.max()
