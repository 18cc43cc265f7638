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
                  and not os.path.basename(p).startswith(("merge_", "v2_")))


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
