"""Generate the golden fixtures in this directory from the reference's own code.

Run in a container that has the reference sources (oracle/ref/Makefile says where it looks;
PDPD_REFERENCE_ROOT overrides it):

    make -C oracle/ref all                           # builds oracle/_ref/ref_harness
    python tests/golden/make_golden.py

The harness (oracle/ref/ref_harness.cpp) compiles the reference's FP64 engines unchanged from
the reference headers.  Each world fixture stores the input world (PDW1 bytes) and the
reference engine's x, v, f after each checkpoint step count, so the tests can run anywhere
without the reference present.  The hash fixture stores get_t_hash / hash_rng_sym /
default_hash outputs of the reference's own functions for seeded and edge-case inputs.
"""

from __future__ import annotations

import io
import os
import struct
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "poets-dpd_gb300"))

import pdpd_world as W  # noqa: E402

HARNESS = os.path.join(ROOT, "oracle", "_ref", "ref_harness")
ENGINE = "naive_dpd_engine_half_step"


def run_reference(world, checkpoints, engine=ENGINE):
    tmp_in = os.path.join(HERE, "_in.pdw1")
    tmp_out = os.path.join(HERE, "_out.bin")
    W.write_pdw1(world, tmp_in)
    # the half-merge engine reports every stationary bead on stderr at each step
    subprocess.run([HARNESS, "step", engine, tmp_in, tmp_out, str(len(checkpoints))]
                   + [str(c) for c in checkpoints], check=True, stderr=subprocess.DEVNULL)
    data = open(tmp_out, "rb").read()
    os.remove(tmp_in)
    os.remove(tmp_out)
    p = 0
    ts, xs, vs, fs = [], [], [], []
    for _ in checkpoints:
        t = int(np.frombuffer(data, np.int64, 1, p)[0])
        n = int(np.frombuffer(data, np.uint32, 1, p + 8)[0])
        p += 12
        rec = np.frombuffer(data, np.float64, 9 * n, p).reshape(n, 9)
        p += 72 * n
        ts.append(t)
        xs.append(rec[:, 0:3])
        vs.append(rec[:, 3:6])
        fs.append(rec[:, 6:9])
    return np.array(ts), np.stack(xs), np.stack(vs), np.stack(fs)


def save_world_fixture(name, world, checkpoints, note, engine=ENGINE):
    ts, xs, vs, fs = run_reference(world, checkpoints, engine)
    buf = io.BytesIO()
    W.write_pdw1(world, buf)
    np.savez_compressed(os.path.join(HERE, name + ".npz"),
                        world=np.frombuffer(buf.getvalue(), np.uint8),
                        checkpoints=np.array(checkpoints), t=ts, x=xs, v=vs, f=fs,
                        engine=np.array(engine), note=np.array(note))
    print(f"{name}: {world.n_beads} beads, checkpoints {checkpoints}")


def pair_world(dx, v0, gamma, box=(4, 4, 4), seed=7):
    """Two monomers at x0 +- dx moving towards each other (a head-on collision)."""
    b = W.WorldBuilder(box, 1, [[25.0]], [[gamma]], dt=0.02, seed=seed)
    b.add_polymer_type([0])
    x0 = np.array([2.0, 2.0, 2.0])
    dx = np.asarray(dx, float)
    b.add_polymer(0, [x0 + dx], [(-np.asarray(v0)).tolist()])
    b.add_polymer(0, [x0 - dx], [np.asarray(v0).tolist()])
    return b.build()


def triple_world(theta0, seed=11):
    """A bent 3-bead chain with Hookean bonds and one angle bond, in a little water."""
    rng = np.random.default_rng(123)
    a, g = W.polymer_interactions(75.0, 4.5)
    b = W.WorldBuilder((5, 5, 5), 3, a, g, dt=0.01, seed=seed)
    b.add_polymer_type([1, 2, 2], [(0, 1, 128.0, 0.5), (1, 2, 128.0, 0.5)],
                       [(0, 1, 20.0, theta0)])
    b.add_polymer_type([0])
    b.add_polymer(0, [(2.0, 2.0, 2.0), (2.45, 2.1, 2.05), (2.7, 2.5, 2.2)],
                  [(0.1, 0.0, 0.0), (0.0, 0.2, 0.0), (0.0, 0.0, -0.1)])
    for _ in range(40):
        b.add_polymer(1, [tuple(rng.random(3) * 5.0)], [tuple(rng.standard_normal(3))])
    return b.build()


def boundary_world(seed=5):
    """Beads placed on cell faces and the box faces, moving across the periodic boundary."""
    b = W.WorldBuilder((4, 4, 4), 1, [[25.0]], [[4.5]], dt=0.02, seed=seed)
    b.add_polymer_type([0])
    pts = [(0.0, 0.0, 0.0), (3.999999999, 2.0, 1.0), (1.0, 3.0, 0.0), (2.0, 2.0, 3.9),
           (0.05, 3.95, 2.0), (3.95, 0.05, 2.0), (1.0, 1.0, 1.0), (2.5, 0.0, 3.5)]
    vel = [(-1.0, -1.0, -1.0), (1.5, 0.0, 0.0), (0.0, 1.0, -2.0), (0.0, 0.0, 3.0),
           (-2.0, 2.0, 0.0), (2.0, -2.0, 0.0), (0.0, 0.0, 0.0), (0.5, -0.5, 0.5)]
    for p, v in zip(pts, vel):
        b.add_polymer(0, [p], [v])
    return b.build()


def stationary_wall_world(seed=13):
    """8^3 water (type 0) against a stationary wall (type 1: the slab 0 <= x < 1, density 3)
    whose beads start with non-zero velocities and forces: they must not move, and their v
    and f are cleared by the first step."""
    rng = np.random.default_rng(77)
    b = W.WorldBuilder((8, 8, 8), 2, [[25.0, 40.0], [40.0, 25.0]], [[4.5, 4.5], [4.5, 4.5]],
                       dt=0.02, seed=seed, stationary=[False, True])
    b.add_polymer_type([0])
    b.add_polymer_type([1])
    for _ in range(3 * 64):
        b.add_polymer(1, [tuple(rng.random(3) * np.array([1.0, 8.0, 8.0]))],
                      [tuple(rng.standard_normal(3))], [tuple(rng.standard_normal(3))])
    for _ in range(3 * 7 * 64):
        b.add_polymer(0, [tuple(np.array([1.0, 0.0, 0.0]) + rng.random(3) * np.array([7.0, 8.0, 8.0]))],
                      [tuple(rng.standard_normal(3))])
    return b.build()


def stationary_anchor_world(seed=17):
    """Chains whose head bead type is stationary (anchored), with Hookean and angle bonds to
    mobile beads, in 8^3 water: bonds across the stationary / mobile boundary."""
    rng = np.random.default_rng(78)
    a = [[25.0, 30.0, 60.0], [30.0, 25.0, 50.0], [60.0, 50.0, 25.0]]
    g = [[4.5] * 3] * 3
    b = W.WorldBuilder((8, 8, 8), 3, a, g, dt=0.01, seed=seed, stationary=[False, True, False])
    b.add_polymer_type([1, 2, 2, 2], [(0, 1, 128.0, 0.5), (1, 2, 128.0, 0.5), (2, 3, 128.0, 0.5)],
                       [(0, 1, 20.0, 0.0), (1, 2, 20.0, 0.0)])
    b.add_polymer_type([0])
    for _ in range(24):
        p0 = rng.random(3) * 8.0
        xs = [p0]
        for _k in range(3):
            d = rng.standard_normal(3)
            xs.append((xs[-1] + 0.5 * d / np.linalg.norm(d)) % 8.0)
        b.add_polymer(0, [tuple(x) for x in xs], [tuple(rng.standard_normal(3)) for _ in xs])
    for _ in range(3 * 512 - 96):
        b.add_polymer(1, [tuple(rng.random(3) * 8.0)], [tuple(rng.standard_normal(3))])
    return b.build()


def permute_bead_ids(world, seed=5):
    """The same world with its bead ids shuffled: polymers then hold non-consecutive ids (the
    v2binary writer's non-sequential bead-id flags)."""
    rng = np.random.default_rng(seed)
    n = world.n_beads
    new_of_old = rng.permutation(n).astype(np.uint32)
    old_of_new = np.argsort(new_of_old)
    w = world.copy()
    for k in ("polymer_id", "polymer_offset", "bead_type", "polymer_type_of_bead", "is_monomer",
              "x", "v", "f"):
        setattr(w, k, getattr(world, k)[old_of_new].copy())
    w.poly_beads = new_of_old[world.poly_beads]
    return w


def v2binary_edge_world():
    """4^3 water whose velocities and forces hit the CVec3Half cases: zero and subnormal
    components, vectors below 2^-14 (encode as zero), exact small integers, mantissas that
    round up to 256 (exponent + 1), ties (round half away from zero), mixed magnitudes;
    positions at 0, at a tie, and just below the box side (rounds to the side: wraps to 0)."""
    w = W.make_water(4, seed=3, gen_seed=5)
    n = w.n_beads
    rng = np.random.default_rng(9)
    special = [
        (0.0, 0.0, 0.0), (5e-324, 0.0, -5e-324), (1e-5, -2e-5, 3e-6), (2.0 ** -15, 0.0, 0.0),
        (2.0 ** -14, 2.0 ** -15, -(2.0 ** -16)), (255.0, -255.0, 17.0), (1.0, 2.0, 3.0),
        (0.9999, 0.5, -0.25), (-0.99999, 0.001, 0.0), (0.5 + 1.0 / 512, 0.0, 0.0),
        (-(0.5 + 1.0 / 512), 0.25 + 1.0 / 1024, 0.0), (32000.0, -1.0, 1e-3),
        (1e4, 1e-9, -1e4), (-3.0e-3, 7.0e-4, 2.5e-3), (0.0, -0.0, 1.0), (-7.5, 0.0, 0.1)]
    v = rng.standard_normal((n, 3)) * np.exp(rng.uniform(-8, 8, (n, 1)))
    f = rng.standard_normal((n, 3)) * np.exp(rng.uniform(-12, 9, (n, 1)))
    for k, s in enumerate(special):
        v[k] = s
        f[len(special) + k] = s
    w.v, w.f = v, f
    x = w.x.copy()
    x[0] = (0.0, 0.0, 0.0)
    x[1] = (1.0 + 0.5 / 65536, 2.0 + 1.5 / 65536, 3.0 - 0.5 / 65536)
    x[2] = (4.0 - 1e-9, 4.0 - 1e-12, 0.5)
    x[3] = (3.9999999, 0.0000001, 2.0)
    w.x = x
    return w


def v2binary_fixture(name, world, note):
    """The reference's own v2binary file of the world (write_world_state, binary) and the
    state its reader returns for that file."""
    tmp_in = os.path.join(HERE, "_v2in.pdw1")
    tmp_v2 = os.path.join(HERE, "_v2.bin")
    tmp_dump = os.path.join(HERE, "_v2.dump")
    W.write_pdw1(world, tmp_in)
    subprocess.run([HARNESS, "v2binary", tmp_in, tmp_v2], check=True)
    subprocess.run([HARNESS, "v2read", tmp_v2, tmp_dump], check=True)
    v2 = open(tmp_v2, "rb").read()
    dump = open(tmp_dump, "rb").read()
    for f in (tmp_in, tmp_v2, tmp_dump):
        os.remove(f)
    n = int(np.frombuffer(dump, np.uint32, 1, 8)[0])
    rec = np.frombuffer(dump, np.float64, 9 * n, 12).reshape(n, 9)
    buf = io.BytesIO()
    W.write_pdw1(world, buf)
    np.savez_compressed(os.path.join(HERE, name + ".npz"),
                        world=np.frombuffer(buf.getvalue(), np.uint8),
                        v2=np.frombuffer(v2, np.uint8), x=rec[:, 0:3], v=rec[:, 3:6], f=rec[:, 6:9],
                        note=np.array(note))
    print(f"{name}: {n} beads, {len(v2)} bytes")


def spatial_fixture(name, world, cons, diss, checkpoints, note, engine="naive_dpd_engine_half_merge"):
    """A world with spatially varying interaction strengths (Parameter expressions, n^2
    conservative and n^2 dissipative strings): the per-cell values the reference evaluates
    (ref_harness tables) and the reference engine's checkpoints (ref_harness stepx)."""
    nt = world.n_types
    tmp_in = os.path.join(HERE, "_sx.pdw1")
    tmp_ex = os.path.join(HERE, "_sx.txt")
    tmp_tab = os.path.join(HERE, "_sx.tab")
    tmp_out = os.path.join(HERE, "_sx.bin")
    W.write_pdw1(world, tmp_in)
    with open(tmp_ex, "w") as fh:
        fh.write("\n".join(list(cons) + list(diss)) + "\n")
    subprocess.run([HARNESS, "tables", tmp_in, tmp_ex, tmp_tab], check=True)
    tab = np.fromfile(tmp_tab, np.float64).reshape(-1, 2, nt, nt)
    subprocess.run([HARNESS, "stepx", engine, tmp_in, tmp_ex, tmp_out, str(len(checkpoints))]
                   + [str(c) for c in checkpoints], check=True, stderr=subprocess.DEVNULL)
    data = open(tmp_out, "rb").read()
    for f in (tmp_in, tmp_ex, tmp_tab, tmp_out):
        os.remove(f)
    p = 0
    ts, xs, vs, fs = [], [], [], []
    for _ in checkpoints:
        t = int(np.frombuffer(data, np.int64, 1, p)[0])
        n = int(np.frombuffer(data, np.uint32, 1, p + 8)[0])
        p += 12
        rec = np.frombuffer(data, np.float64, 9 * n, p).reshape(n, 9)
        p += 72 * n
        ts.append(t)
        xs.append(rec[:, 0:3])
        vs.append(rec[:, 3:6])
        fs.append(rec[:, 6:9])
    buf = io.BytesIO()
    W.write_pdw1(world, buf)
    np.savez_compressed(os.path.join(HERE, name + ".npz"),
                        world=np.frombuffer(buf.getvalue(), np.uint8),
                        checkpoints=np.array(checkpoints), t=np.array(ts), x=np.stack(xs),
                        v=np.stack(vs), f=np.stack(fs), cell_a=tab[:, 0], cell_g=tab[:, 1],
                        exprs=np.array(list(cons) + list(diss)), engine=np.array(engine),
                        note=np.array(note))
    print(f"{name}: {world.n_beads} beads, {tab.shape[0]} cells, checkpoints {checkpoints}")


def hash_fixture():
    rng = np.random.default_rng(2024)
    n = 4096
    t = rng.integers(0, 2**32, n, dtype=np.uint64).astype(np.uint32)
    seed = rng.integers(0, 2**63, n, dtype=np.uint64) * np.uint64(2) + rng.integers(0, 2, n, dtype=np.uint64)
    a = rng.integers(0, 2**32, n, dtype=np.uint64).astype(np.uint32)
    b = rng.integers(0, 2**32, n, dtype=np.uint64).astype(np.uint32)
    edge_t = [0, 1, 0xFFFFFFFF, 0x80000000, 12345]
    edge_s = [0, 1, 0xFFFFFFFFFFFFFFFF, 0x8000000000000000, 42]
    edge_ab = [(0, 0), (1, 0), (0, 1), (0xFFFFFFFF, 0), (0, 0xFFFFFFFF), (0xFFFFFFFF, 0xFFFFFFFF),
               (0x80000000, 0x7FFFFFFF), (7, 7)]
    et, es, ea, eb = [], [], [], []
    for tt in edge_t:
        for ss in edge_s:
            for aa, bb in edge_ab:
                et.append(tt)
                es.append(ss)
                ea.append(aa)
                eb.append(bb)
    t = np.concatenate([t, np.array(et, np.uint32)])
    seed = np.concatenate([seed, np.array(es, np.uint64)])
    a = np.concatenate([a, np.array(ea, np.uint32)])
    b = np.concatenate([b, np.array(eb, np.uint32)])
    rec = np.zeros(t.size, dtype=np.dtype([("t", "<u4"), ("seed", "<u8"), ("a", "<u4"), ("b", "<u4")]))
    rec["t"], rec["seed"], rec["a"], rec["b"] = t, seed, a, b
    tmp_in = os.path.join(HERE, "_hin.bin")
    tmp_out = os.path.join(HERE, "_hout.bin")
    rec.tofile(tmp_in)
    subprocess.run([HARNESS, "hash", tmp_in, tmp_out], check=True)
    out = np.fromfile(tmp_out, dtype=np.dtype([("th", "<u8"), ("h", "<u4"), ("u", "<f4")]))
    os.remove(tmp_in)
    os.remove(tmp_out)
    np.savez_compressed(os.path.join(HERE, "hash_kat.npz"), t=t, seed=seed, a=a, b=b,
                        t_hash=out["th"], h=out["h"], u=out["u"])
    print(f"hash_kat: {t.size} records")


def testbase_fixture(max_segments=4, keep_every_multiple=1):
    """The reference's own engine test suite (225 TestBase cases, test_engine.cpp:62-69),
    driven with the reference's NaiveDPDEngineHalfStep by oracle/ref/testbase_export.cpp.
    Up to max_segments segments per case (the first, the last, evenly spaced ones between);
    keep_every_multiple > 1 thins the 121 TestMultipleMovingBeads cases."""
    exe = os.path.join(ROOT, "oracle", "_ref", "testbase_export")
    tmp = os.path.join(HERE, "_tb.bin")
    subprocess.run([exe, tmp, str(max_segments)], check=True)
    data = open(tmp, "rb").read()
    os.remove(tmp)
    p = 0
    (n,) = struct.unpack_from("<I", data, p)
    p += 4
    names, verdicts, worlds, seg_test, todos, t_in, t_out, s_in, s_out = ([] for _ in range(9))
    multiple_seen = 0
    for _ in range(n):
        (ln,) = struct.unpack_from("<I", data, p)
        p += 4
        name = data[p:p + ln].decode()
        p += ln
        (ok,) = struct.unpack_from("<I", data, p)
        p += 4
        (wl,) = struct.unpack_from("<I", data, p)
        p += 4
        wbytes = data[p:p + wl]
        p += wl
        nb = W.read_pdw1(wbytes).n_beads
        (ns,) = struct.unpack_from("<I", data, p)
        p += 4
        keep = True
        if name.startswith("TestMultipleMovingBeads"):
            keep = multiple_seen % keep_every_multiple == 0
            multiple_seen += 1
        segs = []
        for _ in range(ns):
            (todo,) = struct.unpack_from("<I", data, p)
            p += 4
            (ti,) = struct.unpack_from("<q", data, p)
            p += 8
            xin = np.frombuffer(data, "<f8", 9 * nb, p).reshape(nb, 9)
            p += 72 * nb
            (to,) = struct.unpack_from("<q", data, p)
            p += 8
            xout = np.frombuffer(data, "<f8", 9 * nb, p).reshape(nb, 9)
            p += 72 * nb
            segs.append((todo, ti, xin, to, xout))
        if not keep:
            continue
        k = len(names)
        names.append(name)
        verdicts.append(ok)
        worlds.append(np.frombuffer(wbytes, np.uint8))
        for todo, ti, xin, to, xout in segs:
            seg_test.append(k)
            todos.append(todo)
            t_in.append(ti)
            t_out.append(to)
            s_in.append(xin)
            s_out.append(xout)
    world_off = np.cumsum([0] + [w.size for w in worlds])
    bead_off = np.cumsum([0] + [x.shape[0] for x in s_in])
    np.savez_compressed(os.path.join(HERE, "testbase_suite.npz"),
                        names=np.array(names), verdicts=np.array(verdicts, np.uint8),
                        worlds=np.concatenate(worlds), world_off=world_off,
                        seg_test=np.array(seg_test), todo=np.array(todos), t_in=np.array(t_in),
                        t_out=np.array(t_out), bead_off=bead_off,
                        state_in=np.concatenate(s_in), state_out=np.concatenate(s_out))
    print(f"testbase_suite: {len(names)} of {n} cases, {len(todos)} segments")


PAIR_LOG_NAMES = ["dx", "dr", "dpd-invrootdt", "dpd-gammap", "dpd-rng", "dpd-con", "dpd-diss",
                  "dpd-rng-scale", "dpd-rand", "f_next_dpd"]


def pair_log_fixture(name="pair_log_polymer10", steps=2, ids=(0, 3, 5, 700, 2999)):
    """The reference's per-pair force log (ForceLogging, logging.hpp:9-100, as calc_force makes
    it: dpd_maths_core_half_step.hpp:131-153) of the half-step engine over `steps` steps of
    the 10^3 polymer box, for the listed home beads, at full precision (ref_harness pairlog)."""
    world = W.make_polymer_box(10, chain_fraction=0.1, seed=2)
    tmp_in, tmp_out = os.path.join(HERE, "_in.pdw1"), os.path.join(HERE, "_out.bin")
    W.write_pdw1(world, tmp_in)
    subprocess.run([HARNESS, "pairlog", ENGINE, tmp_in, tmp_out, str(steps), str(len(ids))]
                   + [str(i) for i in ids], check=True)
    data = open(tmp_out, "rb").read()
    os.remove(tmp_in)
    os.remove(tmp_out)
    rec = np.dtype([("t", "<i8"), ("h", "<u4", 2), ("name", "S24"), ("dims", "<i4"), ("v", "<f8", 3)])
    raw = np.frombuffer(data, rec)
    k = len(PAIR_LOG_NAMES)
    assert raw.size % k == 0, raw.size
    names = [n.decode() for n in raw["name"][:k]]
    assert names == PAIR_LOG_NAMES, names
    g = raw.reshape(-1, k)
    assert all((g["name"][:, i] == PAIR_LOG_NAMES[i].encode()).all() for i in range(k))
    out = {"t": g["t"][:, 0], "home_hash": g["h"][:, 0, 0], "other_hash": g["h"][:, 0, 1],
           "dx": g["v"][:, 0], "f": g["v"][:, 9]}
    for i, key in enumerate(["dr", "inv_root_dt", "gammap", "rng", "con", "diss", "rng_scale", "rand"], 1):
        out[key] = g["v"][:, i, 0]
    buf = io.BytesIO()
    W.write_pdw1(world, buf)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), world=np.frombuffer(buf.getvalue(), np.uint8),
                        ids=np.array(ids, np.uint32), steps=np.array(steps), engine=np.array(ENGINE),
                        **out)
    print(f"{name}: {g.shape[0]} pair records of {len(ids)} beads over {steps} steps")


def main():
    if not os.path.exists(HARNESS):
        raise SystemExit("build the reference harness first: make -C oracle/ref")
    if "--only" in sys.argv:  # e.g. --only pair_log: regenerate one fixture
        globals()[sys.argv[sys.argv.index("--only") + 1] + "_fixture"]()
        return
    pair_log_fixture()
    hash_fixture()
    testbase_fixture()
    save_world_fixture("water8_seed1", W.make_water(8, seed=1), [1, 10, 100, 1000],
                       "8^3 water, density 3 (1536 beads), a=25, gamma=4.5, dt=0.02, seed=1 (the reference's "
                       "1000-step FP64 configuration)")
    save_world_fixture("polymer10_seed2", W.make_polymer_box(10, chain_fraction=0.1, seed=2),
                       [1, 10, 50],
                       "10^3 W/H/T polymer-solvent box, 10% in H-T5 chains, k=128 r0=0.5, "
                       "angle k=20 theta0=0, dt=0.01, seed=2")
    save_world_fixture("water_5x7x6_seed3", W.make_water((5, 7, 6), seed=3, gen_seed=33),
                       [1, 10], "non-cubic 5x7x6 water box")
    save_world_fixture("water_3x3x3_seed4", W.make_water(3, seed=4, gen_seed=44), [1, 10],
                       "3^3 box: each neighbour direction wraps onto a distinct cell")
    save_world_fixture("water_2x2x2_seed9", W.make_water(2, seed=9, gen_seed=99), [1, 10],
                       "2^3 box: the -1 and +1 neighbours are the same cell")
    save_world_fixture("pair_conservative", pair_world((0.2, 0, 0), (1.0, 0, 0), 0.0), [1, 10, 40],
                       "head-on pair collision, gamma=0")
    save_world_fixture("pair_dissipative", pair_world((0.15, 0.15, 0.15), (0.5, 0.5, 0.5), 4.5),
                       [1, 10, 40], "diagonal pair collision with dissipation")
    save_world_fixture("triple_angle_theta0", triple_world(0.0), [1, 10, 100],
                       "bent 3-bead chain, angle bond theta0=0, in water")
    save_world_fixture("triple_angle_theta0p2", triple_world(0.2), [1, 10, 100],
                       "bent 3-bead chain, angle bond theta0=0.2 (the sin branch), in water")
    save_world_fixture("boundary_crossing", boundary_world(), [1, 5, 20],
                       "beads on cell and box faces crossing the periodic boundary")
    # Stationary bead types: the half-step engine does not support them
    # (dpd_engine.hpp:86-87), the half-merge engine does (naive_dpd_engine_half_merge.hpp:35);
    # it adds the same pair terms in another order, so these fixtures pin the engine to a
    # tolerance, not bit for bit.
    merge = "naive_dpd_engine_half_merge"
    save_world_fixture("merge_stationary_wall", stationary_wall_world(), [1, 5, 20],
                       "8^3 water against a stationary wall slab (half-merge engine)", merge)
    save_world_fixture("merge_stationary_anchor", stationary_anchor_world(), [1, 5, 20],
                       "chains with stationary heads bonded to mobile beads, in 8^3 water "
                       "(half-merge engine)", merge)
    # Spatially varying interaction strengths (half-merge engine, the one that supports them)
    spatial_fixture("merge_spatial_water", W.make_water(8, seed=6, gen_seed=61),
                    ["25+50*ux"], ["3+3*uy"], [1, 5, 20],
                    "8^3 water, a = 25 + 50 ux, gamma = 3 + 3 uy (half-merge engine)")
    pw = W.make_polymer_box(8, chain_fraction=0.1, seed=7)
    c3 = ["25", "35", "40+40*uz", "35", "25", "75", "40+40*uz", "75", "25-(x-3.5)*(x-3.5)/4"]
    d3 = ["3+3*ux", "4.5", "4.5", "4.5", "4.5", "4.5+y/8", "4.5", "4.5+y/8", "4.5"]
    spatial_fixture("merge_spatial_polymer", pw, c3, d3, [1, 5, 20],
                    "8^3 W/H/T polymer box with a_WT, a_TT, gamma_WW and gamma_HT varying in space "
                    "(half-merge engine)")
    # v2binary snapshots (the reference's writer and reader)
    v2binary_fixture("v2_polymer8", W.make_polymer_box(8, chain_fraction=0.1, seed=2),
                     "8^3 polymer box, 10% H-T5 chains, initial state")
    v2binary_fixture("v2_edges", v2binary_edge_world(), "CVec3Half and position edge cases")
    v2binary_fixture("v2_permuted", permute_bead_ids(W.make_polymer_box(6, chain_fraction=0.3, seed=4)),
                     "6^3 polymer box with shuffled bead ids (non-sequential id records)")
    empty = W.WorldBuilder((4, 4, 4), 1, [[25.0]], [[4.5]], dt=0.02, seed=1)
    empty.add_polymer_type([0])
    save_world_fixture("empty_world", empty.build(), [1, 3], "no beads at all")


if __name__ == "__main__":
    main()
