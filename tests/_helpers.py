"""Shared helpers of the test suite: golden-fixture loading and error metrics."""

from __future__ import annotations

import glob
import os

import numpy as np

import pdpd_world as W

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def world_fixture_names():
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "*.npz"))
                  if not p.endswith("hash_kat.npz"))


def load_world_fixture(name):
    d = np.load(os.path.join(GOLDEN, name + ".npz"))
    world = W.read_pdw1(d["world"].tobytes())
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
