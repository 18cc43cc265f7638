"""The engine library loads and exports every entry point include/pdpd_gpu.h declares; the
host-side validation (CanSupport) works without touching a GPU."""

import os
import re

import numpy as np
import pytest

import pdpd_engine as E
import pdpd_world as W

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _ensure_built():
    if not os.path.exists(E.LIB_PATH):
        import build as B
        B.build()


def header_symbols():
    text = open(os.path.join(ROOT, "include", "pdpd_gpu.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(pdpd_[a-z0-9_]+)\s*\(", text)))


def test_header_and_binding_agree():
    assert sorted(E.EXPORTED) == header_symbols()


def test_library_exports_every_declared_symbol():
    _ensure_built()
    lib = E.lib()
    for name in header_symbols():
        assert hasattr(lib, name), name


def test_can_support_accepts_configs():
    _ensure_built()
    assert E.can_support(W.make_water(8)) == ""
    assert E.can_support(W.make_polymer_box(8, chain_fraction=0.1)) == ""
    assert E.can_support(W.make_water(2)) == ""


def test_can_support_rejections():
    _ensure_built()
    w = W.make_water(4)
    w.stationary = np.array([True])  # supported
    assert E.can_support(w) == ""
    w = W.make_water(4)
    w.box = np.array([4, 1, 4], np.int32)
    assert "at least 2" in E.can_support(w)
    w = W.make_water(4)
    w.dt = 0.0
    assert "dt" in E.can_support(w)
    # 17 bead types do not fit the 4-bit type field of the bead hash
    n = 17
    b = W.WorldBuilder((4, 4, 4), n, np.full((n, n), 25.0), np.full((n, n), 4.5))
    b.add_polymer_type([0])
    b.add_polymer(0, [(1.0, 1.0, 1.0)])
    assert "bead types" in E.can_support(b.build())
    # a bond to a bead that does not exist
    w = W.make_polymer_box(6, chain_fraction=0.1)
    pb = w.poly_beads.copy()  # the topology arrays are read-only: replace one
    pb[1] = w.n_beads + 5
    w.poly_beads = pb
    assert "does not exist" in E.can_support(w)


def test_max_bond_length():
    _ensure_built()
    assert E.lib().pdpd_max_bond_length() == 2.0
