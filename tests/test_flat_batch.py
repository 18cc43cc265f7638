"""The batch attach's struct array (pdpd_engine._flat_batch, built column by column) against
the per-World structs (_Flat): the same scalars, and pointers to the same bytes -- what the
engine reads through them, including its GPU copy kernel reading host memory directly, so a
wrong pointer here must not get as far as a GPU.  CPU only."""

import ctypes as C

import numpy as np

import pdpd_engine as E
import pdpd_world as W

POINTERS = {  # field -> (bytes per element, count field or a number of elements)
    "conservative": 8, "dissipative": 8, "stationary": 1, "hash": 4, "x": 24, "v": 24, "f": 24,
    "bond_beads": 8, "bond_kappa": 8, "bond_r0": 8, "angle_beads": 12, "angle_kappa": 8,
    "angle_theta0": 8, "cell_conservative": 8, "cell_dissipative": 8,
}


def _count(rec, field):
    nt = int(rec["n_bead_types"])
    if field in ("conservative", "dissipative"):
        return nt * nt
    if field == "stationary":
        return nt
    if field in ("hash", "x", "v", "f"):
        return int(rec["n_beads"])
    if field.startswith("bond_"):
        return int(rec["n_bonds"])
    if field.startswith("angle_"):
        return int(rec["n_angles"])
    return int(np.prod(rec["box"])) * nt * nt  # per-cell tables


def _same(a, b):
    for name in E._WORLD_DTYPE.names:
        if name in POINTERS:
            pa, pb = int(a[name]), int(b[name])
            assert (pa == 0) == (pb == 0), name
            if pa:
                n = POINTERS[name] * _count(a, name)
                assert C.string_at(pa, n) == C.string_at(pb, n), name
        else:
            assert np.array_equal(a[name], b[name]), name


def _worlds():
    ws = W.make_batched_grid(512, count=24)
    ws.append(W.make_water(5, seed=3))
    sp = W.make_polymer_box(6, chain_fraction=0.1, seed=4)
    L = sp.box
    nt = sp.conservative.shape[0]
    sp.cell_conservative = np.full((L[0], L[1], L[2], nt, nt), 25.0)
    sp.cell_dissipative = np.full((L[0], L[1], L[2], nt, nt), 4.5)
    ws.append(sp)
    st = W.make_polymer_box(6, chain_fraction=0.1, seed=5)
    st.stationary[0] = True
    st.t = 17
    ws.append(st)
    nc = W.make_water(4, seed=6)
    nc.x = np.asfortranarray(nc.x)  # not C-contiguous: a copy goes to the engine
    ws.append(nc)
    return ws


def test_flat_batch_matches_per_world_structs():
    ws = _worlds()
    arr, keep = E._flat_batch(ws)
    flats = [E._Flat(w) for w in ws]
    ref = np.frombuffer(b"".join(bytes(f.struct) for f in flats), E._WORLD_DTYPE)
    assert arr.dtype == E._WORLD_DTYPE and arr.shape == (len(ws),)
    for i in range(len(ws)):
        _same(arr[i], ref[i])
    del keep


def test_flat_batch_of_copies_reuses_the_topology_part():
    ws = W.make_batched_grid(512, count=4)
    a1, k1 = E._flat_batch(ws)
    a2, k2 = E._flat_batch([w.copy() for w in ws])
    for name in ("hash", "bond_beads", "angle_beads", "n_bonds", "n_angles"):
        assert np.array_equal(a1[name], a2[name])  # the same shared arrays
    assert not np.array_equal(a1["x"], a2["x"])    # the copies' own state
