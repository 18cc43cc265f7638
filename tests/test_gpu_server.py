"""GPU tests of the job server (continuous batching of independent worlds).

Every job's final state must be bit-identical to running its world alone on an engine of the
same precision: the server only changes which worlds share a batch and when, never what a
world computes.  The memory budgets below are chosen so that jobs wait for admission, batches
re-pack as jobs finish, and continuing worlds keep their state on the device across re-packs.
"""

import threading

import numpy as np
import pytest

import pdpd_engine as E
import pdpd_world as W

pytestmark = pytest.mark.gpu


def _jobs():
    """Worlds of mixed size and composition with mixed step counts."""
    out = []
    specs = [(8, 0.05, 30.0, 3.5, 37), (13, 0.05, 80.0, 5.5, 250), (10, 0.0, 55.0, 4.0, 100),
             (9, 0.1, 25.0, 4.5, 163), (12, 0.0, 40.0, 3.0, 1), (8, 0.05, 70.0, 6.0, 299)]
    for i, (L, cf, aw, g, n) in enumerate(specs):
        w = W.make_polymer_box(L, chain_fraction=cf, seed=i + 11, a_wt=aw, gamma=g,
                               gen_seed=300 + i) if cf else W.make_water(L, seed=i + 11, a=aw,
                                                                           gamma=g, gen_seed=300 + i)
        out.append((w, n))
    return out


def _alone(prec, world, n):
    w = world.copy()
    eng = E.GB300DPDEngine(prec)
    eng.Attach(w)
    if n:
        eng.Run(n)
    return w


def _same(a, res):
    x, v, f, t = res
    assert t == a.t
    assert np.array_equal(x, a.x)
    assert np.array_equal(v, a.v)
    assert np.array_equal(f, a.f)


@pytest.mark.parametrize("prec,budget", [("fp32", 1 << 34), ("fp32", 3_000_000), ("fp64", 4_000_000)])
def test_server_jobs_equal_alone(prec, budget):
    jobs = _jobs()
    srv = E.GB300DPDServer(prec, memory_budget_bytes=budget, interval_steps=50)
    ids = [srv.submit(w, n) for w, n in jobs]
    srv.drain()
    st = srv.stats()
    assert st["jobs_done"] == len(jobs) and st["jobs_failed"] == 0
    assert st["bead_steps"] == sum(w.n_beads * n for w, n in jobs)
    assert 0.0 < st["step_s"] <= st["wall_s"]  # device time of the steps, within the wall time
    for jid, (w, n) in zip(ids, jobs):
        _same(_alone(prec, w, n), srv.results[jid])
        assert srv.snapshots.get(jid, 0) == (n - 1) // 50
    if budget < (1 << 30):
        assert st["max_active"] < len(jobs)  # admission control held jobs back
        assert st["repacks"] >= 3
    srv.close()


def test_server_interval_snapshots_and_stop():
    w = W.make_polymer_box(9, chain_fraction=0.05, seed=5, gen_seed=55)
    other = W.make_water(10, seed=6, gen_seed=66)
    seen = []

    def on_interval(jid, t, x, v, f):
        seen.append((t, x, v, f))
        return len(seen) < 3  # stop at the third snapshot

    srv = E.GB300DPDServer("fp32", interval_steps=40)
    j1 = srv.submit(w, 1000, on_interval)
    j2 = srv.submit(other, 200)
    srv.drain()
    assert [s[0] for s in seen] == [w.t + 40, w.t + 80, w.t + 120]
    for k, (t, x, v, f) in enumerate(seen):
        ref = _alone("fp32", w, 40 * (k + 1))
        _same(ref, (x, v, f, t))
    _same(_alone("fp32", w, 120), srv.results[j1])
    _same(_alone("fp32", other, 200), srv.results[j2])
    assert srv.stats()["jobs_done"] == 2
    srv.close()


def test_server_zero_steps_and_submit_from_threads():
    base = [W.make_water(8, seed=20 + i, gen_seed=70 + i) for i in range(6)]
    srv = E.GB300DPDServer("fp32", memory_budget_bytes=2_000_000, interval_steps=30)
    j0 = srv.submit(base[0], 0)
    x, v, f, t = srv.results[j0]
    assert t == base[0].t and np.array_equal(x, base[0].x) and np.array_equal(f, base[0].f)
    ids = {}

    def client(k):
        ids[k] = srv.submit(base[k], 20 * k + 7)

    threads = [threading.Thread(target=client, args=(k,)) for k in range(1, 6)]
    for th in threads:
        th.start()
    for th in threads:
        th.join()
    srv.drain()
    for k in range(1, 6):
        _same(_alone("fp32", base[k], 20 * k + 7), srv.results[ids[k]])
    srv.close()


@pytest.mark.parametrize("prec", ["fp32", "fp64"])
def test_server_failing_job_does_not_disturb_the_others(prec):
    b = W.WorldBuilder((6, 6, 6), 1, [[25.0]], [[4.5]], dt=0.01)
    b.add_polymer_type([0, 0], [(0, 1, 128.0, 0.5)])
    b.add_polymer(0, [(1.0, 1.0, 1.0), (3.5, 1.0, 1.0)])
    bad = b.build()
    good = [W.make_water(8, seed=40 + i, gen_seed=90 + i) for i in range(2)]
    srv = E.GB300DPDServer(prec, interval_steps=25)
    g0 = srv.submit(good[0], 60)
    jb = srv.submit(bad, 60)
    g1 = srv.submit(good[1], 60)
    with pytest.raises(RuntimeError, match="snapped"):
        srv.drain()
    assert srv.failed == {jb: "PDPD_E_BOND_SNAPPED"}
    for jid, w in ((g0, good[0]), (g1, good[1])):
        _same(_alone(prec, w, 60), srv.results[jid])
    st = srv.stats()
    assert st["jobs_done"] == 2 and st["jobs_failed"] == 1
    srv.drain()  # the failure was reported once
    srv.close()


def test_server_config_only_when_idle():
    srv = E.GB300DPDServer("fp32")
    srv.config("force_kernel", 6)
    w = W.make_water(8, seed=3, gen_seed=33)
    j = srv.submit(w, 30)
    srv.drain()
    _same(_alone("fp32", w, 30), srv.results[j])
    with pytest.raises(RuntimeError, match="unknown|Unknown|not"):
        srv.config("no_such_key", 1)
    srv.close()
