"""Shared helpers of the test suite: golden-fixture loading and error metrics."""

from __future__ import annotations

import glob
import os

import numpy as np

import pdpd_world as W

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def world_fixture_names():
    """Fixtures made by the reference's half-step engine (the FP64 engine matches them bit for
    bit)."""
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "*.npz"))
                  if not p.endswith(("hash_kat.npz", "testbase_suite.npz"))
                  and not os.path.basename(p).startswith(("merge_", "v2_", "pair_log_")))


def merge_fixture_names(kind=""):
    """Fixtures made by the reference's half-merge engine (worlds with stationary bead types or
    spatially varying strengths, which the half-step engine does not support): same terms,
    another summation order.  kind: "stationary", "spatial" or "" (all)."""
    return sorted(os.path.basename(p)[:-4]
                  for p in glob.glob(os.path.join(GOLDEN, f"merge_{kind}*.npz")))


def state_rel_err(a, b):
    """max |a - b| / rms |b| over all beads and components (0 when both are zero)."""
    scale = np.sqrt(np.mean(np.sum(b * b, axis=1))) if b.size else 0.0
    d = np.max(np.abs(a - b)) if b.size else 0.0
    return 0.0 if d == 0 else float(d / max(scale, 1e-300))


def load_world_fixture(name):
    d = np.load(os.path.join(GOLDEN, name + ".npz"))
    world = W.read_pdw1(d["world"].tobytes())
    if "cell_a" in d.files:  # spatially varying strengths, as the reference evaluated them
        world.cell_conservative = d["cell_a"].copy()
        world.cell_dissipative = d["cell_g"].copy()
    return world, {k: d[k] for k in ("checkpoints", "t", "x", "v", "f")}


def load_hash_kat():
    d = np.load(os.path.join(GOLDEN, "hash_kat.npz"))
    return {k: d[k] for k in d.files}


def periodic_dx(a, b, box):
    d = a - b
    L = np.asarray(box, float)[None, :]
    return d - L * np.round(d / L)


def force_rel_err(f, f_ref):
    """max_i |f_i - f_ref_i| / rms_j |f_ref_j|: the largest per-bead force error relative to the
    force scale of the world (single beads can have a near-zero net force)."""
    if f_ref.size == 0:
        return 0.0
    scale = np.sqrt(np.mean(np.sum(f_ref * f_ref, axis=1)))
    scale = max(scale, 1e-300)
    return float(np.max(np.linalg.norm(f - f_ref, axis=1)) / scale)


# Worst-case error of one pair's separation in the FP32 engine after one step: each stored
# position offset (in [0, 1)) is rounded to FP32 at attach and again by update_pos, <= 2^-25
# each per axis, and the separation is rounded once (<= 2^-24 of a value below 1), so per axis
# <= 3 * 2^-24 and over three axes <= sqrt(3) * 3 * 2^-24 < 2^-21.
FP32_SEP_ERR = 2.0 ** -21


def fp32_force_check(world, x, v, f, f_ref, tol=1e-5, r_close=0.01, slack=10.0):
    """One-step FP32 forces against FP64 ones: every bead within tol * rms|f_ref|, except a
    bead with a pair closer than r_close, whose unit vector the FP32 storage of positions
    alone turns by up to FP32_SEP_ERR / r.  Such a bead may reach slack * tol * rms|f_ref|,
    and no more than the storage error carried through its close pairs: the sum over them of
    F_max (4 / r + 2) FP32_SEP_ERR, where F_max = a_max + gamma_max (|v_i - v_j| + 1) +
    sqrt(gamma_max) sqrt(24 / dt) / 2 bounds the pair force and its r-derivative / 2.  Such
    beads must also be rare: at most 1e-5 of the beads + 2.  x, v: the positions the forces
    were evaluated at and the velocities (FP64 run).  Returns (max error / rms, beads above
    tol)."""
    scale = np.sqrt(np.mean(np.sum(f_ref * f_ref, axis=1)))
    err = np.linalg.norm(f - f_ref, axis=1)
    bad = np.nonzero(err > tol * scale)[0]
    assert len(bad) <= 1e-5 * len(err) + 2, f"{len(bad)} beads above {tol:g} of rms|f|"
    a_max, g_max = float(world.conservative.max()), float(world.dissipative.max())
    rand = np.sqrt(g_max) * np.sqrt(24.0 / world.dt) / 2
    L = np.asarray(world.box, float)
    for i in bad:
        d = x - x[i]
        d -= L * np.round(d / L)
        r = np.linalg.norm(d, axis=1)
        m = (r < r_close) & (r > 0.0)
        assert m.any(), (int(i), float(err[i] / scale), "no pair closer than", r_close)
        f_max = a_max + g_max * (np.linalg.norm(v[m] - v[i], axis=1) + 1.0) + rand
        bound = min(slack * tol * scale, np.sum(f_max * (4.0 / r[m] + 2.0)) * FP32_SEP_ERR)
        assert err[i] <= bound, (int(i), float(err[i]), float(bound), float(r[m].min()))
    return float(err.max() / scale) if err.size else 0.0, len(bad)


def load_testbase():
    """The reference's TestBase suite as replayable segments (tests/golden/testbase_suite.npz):
    a list of (name, world, [(todo, t_in, state_in (n,9), t_out, state_out (n,9)), ...]) where a
    state row is x, v, f of one bead."""
    d = np.load(os.path.join(GOLDEN, "testbase_suite.npz"))
    cases = []
    names = d["names"]
    segs_of = {}
    for s, k in enumerate(d["seg_test"]):
        segs_of.setdefault(int(k), []).append(s)
    bo, wo = d["bead_off"], d["world_off"]
    for k, name in enumerate(names):
        world = W.read_pdw1(d["worlds"][wo[k]:wo[k + 1]].tobytes())
        segs = []
        for s in segs_of.get(k, []):
            segs.append((int(d["todo"][s]), int(d["t_in"][s]), d["state_in"][bo[s]:bo[s + 1]],
                         int(d["t_out"][s]), d["state_out"][bo[s]:bo[s + 1]]))
        cases.append((str(name), world, segs))
    return cases


def world_at(world, t, state):
    """Copy of world with time t and bead state rows (x, v, f)."""
    w = world.copy()
    w.t = t
    w.x, w.v, w.f = state[:, 0:3].copy(), state[:, 3:6].copy(), state[:, 6:9].copy()
    return w


def v2_fixture_names():
    """v2binary fixtures: a world, the reference's v2binary file of it, and the state the
    reference's reader returns for that file."""
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "v2_*.npz")))


def load_v2_fixture(name):
    d = np.load(os.path.join(GOLDEN, name + ".npz"))
    return W.read_pdw1(d["world"].tobytes()), d["v2"].tobytes(), d["x"], d["v"], d["f"]
