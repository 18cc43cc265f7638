"""Host-side mirror of the reference's ``WorldState`` (include/dpd/core/dpd_state.hpp:245-264).

A :class:`World` holds the same information as a ``WorldState``: box, dt, lambda, seed, t,
the bead-type interaction matrix, polymer types with Hookean bonds and angle bond pairs,
polymers, and per-bead identity and x/v/f.  It is stored as numpy arrays rather than an
array of ``Bead`` structs so it can be handed to the engine's C ABI without copying.

Also here:

* ``bead_hash`` -- the 32-bit ``BeadHash::construct`` encoding (dpd_state.hpp:52-60).
* ``flat_bonds`` -- the polymer/bond templates expanded into flat per-bond and per-angle
  lists, in the order the reference engines visit them (polymer by polymer, bonds in
  polymer-type order, then bond pairs in polymer-type order;
  naive_dpd_engine_half_step.hpp:321-329).
* generators for the synthetic worlds the engine is tested and measured on (water boxes,
  polymer-solvent boxes, batched grids), seeded, using numpy only.
* the PDW1 binary world file format, shared with the C++ test harnesses under oracle/ref/.
"""

from __future__ import annotations

import math
import struct
from dataclasses import dataclass, field

import numpy as np

# BeadHash layout (dpd_state.hpp:18-40): bbbb 1ppp...p (monomer, 27-bit id) or
# bbbb 0ooo oooo pppp...p (polymer bead: 7-bit offset, 20-bit polymer id).
MONOMER_ID_BITS = 27
POLYMER_ID_BITS = 20
BEAD_TYPE_SHIFT = 28
MONOMER_FLAG_SHIFT = 27
POLYMER_OFFSET_SHIFT = 20
MAX_BEAD_TYPES = 16
MAX_POLYMER_OFFSET = 127


def bead_hash(bead_type, is_monomer, polymer_id, polymer_offset):
    """Vectorised ``BeadHash::construct`` (dpd_state.hpp:52-60)."""
    # 32-bit arithmetic: bits shifted past bit 31 are dropped, as in the 32-bit hash
    h = np.asarray(polymer_offset).astype(np.uint32) << np.uint32(POLYMER_OFFSET_SHIFT)
    h |= np.asarray(polymer_id).astype(np.uint32)
    h |= np.asarray(is_monomer).astype(np.uint32) << np.uint32(MONOMER_FLAG_SHIFT)
    h |= np.asarray(bead_type).astype(np.uint32) << np.uint32(BEAD_TYPE_SHIFT)
    return h


@dataclass
class PolymerType:
    """``PolymerType`` (dpd_state.hpp:212-224) with constant bond parameters."""

    bead_types: list
    bonds: list = field(default_factory=list)        # (head_offset, tail_offset, kappa, r0)
    bond_pairs: list = field(default_factory=list)   # (head_bond, tail_bond, kappa, theta0)


# The bead and polymer topology of a World: fixed once the World is built, as the reference
# keeps a WorldState's types and polymers fixed while it is attached (dpd_engine.hpp:171-176).
# These arrays are stored read-only (an assignment replaces one), so the arrays derived from
# them -- the bead hashes and the flat bond lists, which every attach needs -- are computed
# once and shared by the World's copies.
_TOPOLOGY = ("poly_type", "poly_start", "poly_beads", "polymer_id", "polymer_offset", "bead_type",
             "polymer_type_of_bead", "is_monomer")


def _read_only(a):
    if isinstance(a, np.ndarray) and not a.flags.writeable:
        return a
    v = np.asarray(a).view()
    v.flags.writeable = False
    return v


@dataclass
class World:
    box: np.ndarray                 # (3,) int32 box sides
    dt: float
    lam: float
    seed: int
    t: int
    conservative: np.ndarray        # (nt, nt) a_ij
    dissipative: np.ndarray         # (nt, nt) gamma_ij
    stationary: np.ndarray          # (nt,) bool
    polymer_types: list
    poly_type: np.ndarray           # (np,) uint32
    poly_start: np.ndarray          # (np+1,) uint32: CSR into poly_beads
    poly_beads: np.ndarray          # bead ids of each polymer, in offset order
    polymer_id: np.ndarray          # (n,) uint32
    polymer_offset: np.ndarray      # (n,) uint8
    bead_type: np.ndarray           # (n,) uint8
    polymer_type_of_bead: np.ndarray  # (n,) uint8
    is_monomer: np.ndarray          # (n,) bool
    x: np.ndarray                   # (n, 3) float64
    v: np.ndarray
    f: np.ndarray
    # spatially varying strengths: per cell (x-major, z fastest) (nt, nt) a_ij and gamma_ij,
    # or None (the matrices above everywhere)
    cell_conservative: np.ndarray = None
    cell_dissipative: np.ndarray = None

    @property
    def n_beads(self) -> int:
        return int(self.x.shape[0])

    @property
    def n_types(self) -> int:
        return int(self.conservative.shape[0])

    def __post_init__(self):
        # the bead hashes and bond lists of a new topology, once (its copies share them)
        self.hashes()
        self.flat_bonds()

    def __setattr__(self, name, value):
        if name in _TOPOLOGY and value is not None:
            value = _read_only(value)
        object.__setattr__(self, name, value)

    def _derived(self, what, fields, extra, make):
        """make(), cached while the named topology arrays are the same objects (they are
        read-only) and `extra` compares equal."""
        cache = self.__dict__.setdefault("_cache", {})
        arrays = tuple(getattr(self, k) for k in fields)
        hit = cache.get(what)
        if hit is not None and hit[1] == extra and all(a is b for a, b in zip(hit[0], arrays)):
            return hit[2]
        value = make()
        value = tuple(_read_only(v) for v in value) if isinstance(value, tuple) else _read_only(value)
        cache[what] = (arrays, extra, value)
        return value

    def hashes(self) -> np.ndarray:
        """BeadHash of every bead (read-only; computed once per topology)."""
        return self._derived("hash", ("bead_type", "is_monomer", "polymer_id", "polymer_offset"), None,
                             lambda: bead_hash(self.bead_type, self.is_monomer, self.polymer_id,
                                               self.polymer_offset))

    def copy(self) -> "World":
        """A copy with its own state (x, v, f, t, parameters); the read-only topology arrays
        and what is derived from them (the hashes, the flat bond lists, the C ABI's topology
        struct) are shared."""
        w = World(
            box=self.box.copy(), dt=self.dt, lam=self.lam, seed=self.seed, t=self.t,
            conservative=self.conservative.copy(), dissipative=self.dissipative.copy(),
            stationary=self.stationary.copy(),
            polymer_types=[PolymerType(list(p.bead_types), list(p.bonds), list(p.bond_pairs))
                           for p in self.polymer_types],
            poly_type=self.poly_type, poly_start=self.poly_start, poly_beads=self.poly_beads,
            polymer_id=self.polymer_id, polymer_offset=self.polymer_offset, bead_type=self.bead_type,
            polymer_type_of_bead=self.polymer_type_of_bead, is_monomer=self.is_monomer,
            x=self.x.copy(), v=self.v.copy(), f=self.f.copy(),
            cell_conservative=None if self.cell_conservative is None else self.cell_conservative.copy(),
            cell_dissipative=None if self.cell_dissipative is None else self.cell_dissipative.copy())
        # one cache for a World and all its copies: an entry is used only while the topology
        # arrays it was made from are the ones of the World asking, so a copy whose topology
        # was replaced recomputes (and the others recompute after it)
        w.__dict__["_cache"] = self.__dict__.setdefault("_cache", {})
        return w

    def flat_bonds(self):
        """Expand the polymer templates into flat bond and angle lists (read-only; computed
        once per topology and polymer types).

        Returns ``(bond_beads (nb,2) uint32, bond_kappa, bond_r0, angle_beads (na,3) uint32,
        angle_kappa, angle_theta0)``.  Order: polymers in id order; within a polymer, bonds in
        polymer-type order; all Hookean bonds come before all angle bonds.  Each bead belongs
        to one polymer, so each bead sees its bond terms in the same order as the reference's
        per-polymer loop (naive_dpd_engine_half_step.hpp:321-329).
        """
        types = tuple((tuple(p.bead_types), tuple(map(tuple, p.bonds)), tuple(map(tuple, p.bond_pairs)))
                      for p in self.polymer_types)
        return self._derived("bonds", ("poly_type", "poly_start", "poly_beads"), types, self._expand_bonds)

    def _expand_bonds(self):
        bonds = {"beads": [], "kappa": [], "r0": [], "poly": []}
        angles = {"beads": [], "kappa": [], "theta0": [], "poly": []}
        with_terms = [i for i, pt in enumerate(self.polymer_types) if pt.bonds or pt.bond_pairs]
        # one polymer type with bond terms: its polymers, in id order, give the lists in order
        single = len(with_terms) == 1
        for pt_index in with_terms:
            pt = self.polymer_types[pt_index]
            sel = (np.arange(self.poly_type.shape[0]) if len(self.polymer_types) == 1
                   else np.nonzero(self.poly_type == pt_index)[0])
            if sel.size == 0:
                continue
            starts = self.poly_start[sel].astype(np.int64)
            if pt.bonds:
                ht = np.array([[b[0], b[1]] for b in pt.bonds], dtype=np.int64)  # (bonds, 2)
                bonds["beads"].append(self.poly_beads[starts[:, None, None] + ht[None, :, :]].reshape(-1, 2))
                bonds["kappa"].append(np.tile(np.array([b[2] for b in pt.bonds], float), sel.size))
                bonds["r0"].append(np.tile(np.array([b[3] for b in pt.bonds], float), sel.size))
                if not single:
                    bonds["poly"].append(np.repeat(sel, len(pt.bonds)))
            if pt.bond_pairs:
                hmt = np.array([[pt.bonds[q[0]][0], pt.bonds[q[0]][1], pt.bonds[q[1]][1]]
                                for q in pt.bond_pairs], dtype=np.int64)  # (pairs, 3)
                angles["beads"].append(self.poly_beads[starts[:, None, None] + hmt[None, :, :]].reshape(-1, 3))
                angles["kappa"].append(
                    np.tile(np.array([q[2] for q in pt.bond_pairs], float), sel.size))
                angles["theta0"].append(
                    np.tile(np.array([q[3] for q in pt.bond_pairs], float), sel.size))
                if not single:
                    angles["poly"].append(np.repeat(sel, len(pt.bond_pairs)))

        def finish(d, width, keys):
            if not d["beads"]:
                return [np.zeros((0, width), np.uint32)] + [np.zeros(0) for _ in keys]
            if len(d["beads"]) == 1:  # one polymer type: already in polymer id order
                return ([np.ascontiguousarray(d["beads"][0], dtype=np.uint32)] +
                        [np.ascontiguousarray(d[k][0], dtype=np.float64) for k in keys])
            order = np.argsort(np.concatenate(d["poly"]), kind="stable")
            out = [np.concatenate(d["beads"]).astype(np.uint32)[order]]
            out += [np.concatenate(d[k]).astype(np.float64)[order] for k in keys]
            return out

        bb, bk, br = finish(bonds, 2, ["kappa", "r0"])
        ab, ak, at = finish(angles, 3, ["kappa", "theta0"])
        return bb, bk, br, ab, ak, at


# ---------------------------------------------------------------------------------------
# Builders
# ---------------------------------------------------------------------------------------

class WorldBuilder:
    """Incremental builder in the spirit of ``WorldStateBuilder`` (dpd_state_builder.hpp:18-232):
    bead ids and polymer ids are assigned in insertion order."""

    def __init__(self, box, n_types, conservative, dissipative, dt=0.02, lam=0.5, seed=1, t=0,
                 stationary=None):
        self.box = np.asarray(box, dtype=np.int32)
        self.conservative = np.asarray(conservative, float).reshape(n_types, n_types)
        self.dissipative = np.asarray(dissipative, float).reshape(n_types, n_types)
        self.stationary = np.zeros(n_types, bool) if stationary is None else np.asarray(stationary, bool)
        self.dt, self.lam, self.seed, self.t = dt, lam, seed, t
        self.polymer_types: list = []
        self.polymers: list = []   # (type, [bead ids])
        self.beads: list = []      # (polymer_id, offset, type, ptype, is_monomer, x, v, f)

    def add_polymer_type(self, bead_types, bonds=(), bond_pairs=()):
        self.polymer_types.append(PolymerType(list(bead_types), list(bonds), list(bond_pairs)))
        return len(self.polymer_types) - 1

    def add_polymer(self, ptype, xs, vs=None, fs=None):
        pt = self.polymer_types[ptype]
        pid = len(self.polymers)
        ids = []
        for i, x in enumerate(xs):
            v = (0.0, 0.0, 0.0) if vs is None else vs[i]
            f = (0.0, 0.0, 0.0) if fs is None else fs[i]
            ids.append(len(self.beads))
            self.beads.append((pid, i, pt.bead_types[i], ptype, len(pt.bead_types) == 1, x, v, f))
        self.polymers.append((ptype, ids))
        return pid

    def build(self) -> World:
        n = len(self.beads)
        poly_type = np.array([p[0] for p in self.polymers], np.uint32)
        sizes = np.array([len(p[1]) for p in self.polymers], np.int64)
        poly_start = np.zeros(len(self.polymers) + 1, np.uint32)
        poly_start[1:] = np.cumsum(sizes)
        poly_beads = np.array([i for p in self.polymers for i in p[1]], np.uint32)
        col = lambda k, dt: np.array([b[k] for b in self.beads], dtype=dt)
        vec = lambda k: np.array([b[k] for b in self.beads], dtype=np.float64).reshape(n, 3)
        return World(
            box=self.box.copy(), dt=self.dt, lam=self.lam, seed=self.seed, t=self.t,
            conservative=self.conservative.copy(), dissipative=self.dissipative.copy(),
            stationary=self.stationary.copy(), polymer_types=self.polymer_types,
            poly_type=poly_type, poly_start=poly_start, poly_beads=poly_beads,
            polymer_id=col(0, np.uint32), polymer_offset=col(1, np.uint8),
            bead_type=col(2, np.uint8), polymer_type_of_bead=col(3, np.uint8),
            is_monomer=col(4, bool), x=vec(5), v=vec(6), f=vec(7))


TYPE_W, TYPE_H, TYPE_T = 0, 1, 2
CHAIN_TYPES = [TYPE_H, TYPE_T, TYPE_T, TYPE_T, TYPE_T, TYPE_T]


def _gaussian_velocities(rng, n):
    v = rng.standard_normal((n, 3))
    if n > 1:
        v -= v.mean(axis=0, keepdims=True)
    return v


def make_water(L, seed=1, a=25.0, gamma=4.5, dt=0.02, density=3, gen_seed=None, t=0):
    """Pure DPD water in a periodic L^3 cube: density*L^3 beads of one type, uniform random
    positions, Gaussian kT=1 velocities with the net momentum removed, f = 0."""
    rng = np.random.default_rng(seed if gen_seed is None else gen_seed)
    Ls = np.array([L, L, L] if np.isscalar(L) else L, np.int32)
    n = int(density * int(np.prod(Ls.astype(np.int64))))
    x = rng.random((n, 3)) * Ls[None, :]
    x = np.where(x >= Ls[None, :], 0.0, x)
    v = _gaussian_velocities(rng, n)
    return _assemble_monomer_world(Ls, x, v, np.array([[a]]), np.array([[gamma]]), dt, seed, t,
                                   n_types=1)


def _assemble_monomer_world(Ls, x, v, cons, diss, dt, seed, t, n_types):
    n = x.shape[0]
    return World(
        box=Ls, dt=dt, lam=0.5, seed=seed, t=t, conservative=cons.astype(float),
        dissipative=diss.astype(float), stationary=np.zeros(n_types, bool),
        polymer_types=[PolymerType([0])], poly_type=np.zeros(n, np.uint32),
        poly_start=np.arange(n + 1, dtype=np.uint32), poly_beads=np.arange(n, dtype=np.uint32),
        polymer_id=np.arange(n, dtype=np.uint32), polymer_offset=np.zeros(n, np.uint8),
        bead_type=np.zeros(n, np.uint8), polymer_type_of_bead=np.zeros(n, np.uint8),
        is_monomer=np.ones(n, bool), x=x, v=v, f=np.zeros((n, 3)))


def polymer_interactions(a_wt=75.0, gamma=4.5):
    """3-type W/H/T matrix: a_WW=a_HH=a_TT=25, a_WH=35, a_WT=a_wt, a_HT=75; gamma everywhere."""
    a = np.array([[25.0, 35.0, a_wt],
                  [35.0, 25.0, 75.0],
                  [a_wt, 75.0, 25.0]])
    g = np.full((3, 3), float(gamma))
    return a, g


def make_polymer_box(L, chain_fraction=0.1, seed=2, a_wt=75.0, gamma=4.5, dt=0.01,
                     kappa_bond=128.0, r0=0.5, kappa_angle=20.0, theta0=0.0, density=3,
                     gen_seed=None, t=0):
    """Polymer-solvent box: density*L^3 beads, floor(chain_fraction*N/6) linear H-T-T-T-T-T
    chains (added first, so chain polymer ids stay below 2^20) and W monomers for the rest.

    Chains: Hookean bonds (kappa_bond, r0) between consecutive beads, angle bonds
    (kappa_angle, theta0) on consecutive bond pairs.  The first bead of a chain is uniform in
    the box, each next bead is r0 away in a uniformly random direction (wrapped).
    """
    rng = np.random.default_rng(seed if gen_seed is None else gen_seed)
    Ls = np.array([L, L, L] if np.isscalar(L) else L, np.int32)
    Lf = Ls.astype(np.float64)
    n = int(density * int(np.prod(Ls.astype(np.int64))))
    n_chains = int(math.floor(chain_fraction * n / 6))
    n_chain_beads = 6 * n_chains
    n_mono = n - n_chain_beads
    x = np.empty((n, 3))
    if n_chains:
        cx = np.empty((n_chains, 6, 3))
        cx[:, 0] = rng.random((n_chains, 3)) * Lf
        for k in range(1, 6):
            d = rng.standard_normal((n_chains, 3))
            d /= np.linalg.norm(d, axis=1, keepdims=True)
            cx[:, k] = cx[:, k - 1] + r0 * d
        cx = np.mod(cx, Lf)
        cx = np.where(cx >= Lf, 0.0, cx)
        x[:n_chain_beads] = cx.reshape(-1, 3)
    xm = rng.random((n_mono, 3)) * Lf
    x[n_chain_beads:] = np.where(xm >= Lf, 0.0, xm)
    v = _gaussian_velocities(rng, n)
    a, g = polymer_interactions(a_wt, gamma)

    chain_type = PolymerType(
        list(CHAIN_TYPES),
        [(i, i + 1, kappa_bond, r0) for i in range(5)],
        [(i, i + 1, kappa_angle, theta0) for i in range(4)])
    water_type = PolymerType([TYPE_W])
    n_poly = n_chains + n_mono
    poly_type = np.concatenate([np.zeros(n_chains, np.uint32), np.ones(n_mono, np.uint32)])
    sizes = np.concatenate([np.full(n_chains, 6, np.int64), np.ones(n_mono, np.int64)])
    poly_start = np.zeros(n_poly + 1, np.uint32)
    poly_start[1:] = np.cumsum(sizes)
    polymer_id = np.concatenate([np.repeat(np.arange(n_chains, dtype=np.uint32), 6),
                                 np.arange(n_chains, n_poly, dtype=np.uint32)])
    polymer_offset = np.concatenate([np.tile(np.arange(6, dtype=np.uint8), n_chains),
                                     np.zeros(n_mono, np.uint8)])
    bead_type = np.concatenate([np.tile(np.array(CHAIN_TYPES, np.uint8), n_chains),
                                np.full(n_mono, TYPE_W, np.uint8)])
    ptype_of_bead = np.concatenate([np.zeros(n_chain_beads, np.uint8), np.ones(n_mono, np.uint8)])
    is_monomer = np.concatenate([np.zeros(n_chain_beads, bool), np.ones(n_mono, bool)])
    return World(
        box=Ls, dt=dt, lam=0.5, seed=seed, t=t, conservative=a, dissipative=g,
        stationary=np.zeros(3, bool), polymer_types=[chain_type, water_type],
        poly_type=poly_type, poly_start=poly_start, poly_beads=np.arange(n, dtype=np.uint32),
        polymer_id=polymer_id, polymer_offset=polymer_offset, bead_type=bead_type,
        polymer_type_of_bead=ptype_of_bead, is_monomer=is_monomer, x=x, v=v, f=np.zeros((n, 3)))


def make_batched_grid(n_states=512, side_lo=8, side_hi=32, chain_fraction=0.05, steps=200,
                      gen_seed=4, count=None):
    """Batched grid of independent polymer-solvent states: cube side uniform on
    [side_lo, side_hi], per-state a_WT ~ U[25,100], gamma ~ U[3,6] (all pairs), state seed
    = index+1, dt = 0.01.  ``count`` builds only the first ``count`` states (the same ones the
    full grid starts with)."""
    rng = np.random.default_rng(gen_seed)
    sides = rng.integers(side_lo, side_hi + 1, size=n_states)
    a_wt = rng.uniform(25.0, 100.0, size=n_states)
    gam = rng.uniform(3.0, 6.0, size=n_states)
    worlds = []
    for i in range(n_states if count is None else min(count, n_states)):
        worlds.append(make_polymer_box(int(sides[i]), chain_fraction=chain_fraction, seed=i + 1,
                                       a_wt=float(a_wt[i]), gamma=float(gam[i]), dt=0.01,
                                       gen_seed=gen_seed * 100003 + i))
    return worlds


# ---------------------------------------------------------------------------------------
# PDW1 file format
# ---------------------------------------------------------------------------------------

def write_pdw1(world: World, path_or_file):
    out = bytearray()
    out += b"PDW1"
    out += struct.pack("<3i", *[int(b) for b in world.box])
    out += struct.pack("<ddQq", world.dt, world.lam, world.seed & 0xFFFFFFFFFFFFFFFF, world.t)
    nt = world.n_types
    out += struct.pack("<I", nt)
    out += np.asarray(world.stationary, np.uint32).tobytes()
    out += np.asarray(world.conservative, "<f8").reshape(-1).tobytes()
    out += np.asarray(world.dissipative, "<f8").reshape(-1).tobytes()
    out += struct.pack("<I", len(world.polymer_types))
    for pt in world.polymer_types:
        out += struct.pack("<I", len(pt.bead_types))
        out += np.asarray(pt.bead_types, "<u4").tobytes()
        out += struct.pack("<I", len(pt.bonds))
        for h, t, k, r0 in pt.bonds:
            out += struct.pack("<IIdd", h, t, k, r0)
        out += struct.pack("<I", len(pt.bond_pairs))
        for h, t, k, th in pt.bond_pairs:
            out += struct.pack("<IIdd", h, t, k, th)
    npoly = len(world.poly_type)
    out += struct.pack("<I", npoly)
    sizes = np.diff(world.poly_start.astype(np.int64))
    for i in range(npoly):
        out += struct.pack("<II", int(world.poly_type[i]), int(sizes[i]))
        out += world.poly_beads[world.poly_start[i]:world.poly_start[i + 1]].astype("<u4").tobytes()
    n = world.n_beads
    out += struct.pack("<I", n)
    rec = np.zeros(n, dtype=np.dtype([("id", "<u4"), ("pid", "<u4"), ("off", "u1"), ("bt", "u1"),
                                      ("pt", "u1"), ("mono", "u1"), ("x", "<f8", 3),
                                      ("v", "<f8", 3), ("f", "<f8", 3)]))
    rec["id"] = np.arange(n)
    rec["pid"] = world.polymer_id
    rec["off"] = world.polymer_offset
    rec["bt"] = world.bead_type
    rec["pt"] = world.polymer_type_of_bead
    rec["mono"] = world.is_monomer
    rec["x"], rec["v"], rec["f"] = world.x, world.v, world.f
    out += rec.tobytes()
    if hasattr(path_or_file, "write"):
        path_or_file.write(bytes(out))
    else:
        with open(path_or_file, "wb") as fh:
            fh.write(bytes(out))


def read_pdw1(data) -> World:
    if not isinstance(data, (bytes, bytearray)):
        with open(data, "rb") as fh:
            data = fh.read()
    mv = memoryview(data)
    assert bytes(mv[:4]) == b"PDW1", "not a PDW1 file"
    p = 4
    box = np.array(struct.unpack_from("<3i", mv, p), np.int32); p += 12
    dt, lam, seed, t = struct.unpack_from("<ddQq", mv, p); p += 32
    (nt,) = struct.unpack_from("<I", mv, p); p += 4
    stationary = np.frombuffer(mv, "<u4", nt, p).astype(bool); p += 4 * nt
    cons = np.frombuffer(mv, "<f8", nt * nt, p).reshape(nt, nt).copy(); p += 8 * nt * nt
    diss = np.frombuffer(mv, "<f8", nt * nt, p).reshape(nt, nt).copy(); p += 8 * nt * nt
    (npt,) = struct.unpack_from("<I", mv, p); p += 4
    pts = []
    for _ in range(npt):
        (nb,) = struct.unpack_from("<I", mv, p); p += 4
        bts = list(np.frombuffer(mv, "<u4", nb, p)); p += 4 * nb
        (nbond,) = struct.unpack_from("<I", mv, p); p += 4
        bonds = []
        for _ in range(nbond):
            bonds.append(struct.unpack_from("<IIdd", mv, p)); p += 24
        (npair,) = struct.unpack_from("<I", mv, p); p += 4
        pairs = []
        for _ in range(npair):
            pairs.append(struct.unpack_from("<IIdd", mv, p)); p += 24
        pts.append(PolymerType([int(b) for b in bts], bonds, pairs))
    (npoly,) = struct.unpack_from("<I", mv, p); p += 4
    poly_type = np.zeros(npoly, np.uint32)
    poly_start = np.zeros(npoly + 1, np.uint32)
    beads = []
    for i in range(npoly):
        ptype, sz = struct.unpack_from("<II", mv, p); p += 8
        poly_type[i] = ptype
        beads.append(np.frombuffer(mv, "<u4", sz, p)); p += 4 * sz
        poly_start[i + 1] = poly_start[i] + sz
    poly_beads = np.concatenate(beads).astype(np.uint32) if beads else np.zeros(0, np.uint32)
    (n,) = struct.unpack_from("<I", mv, p); p += 4
    dtype = np.dtype([("id", "<u4"), ("pid", "<u4"), ("off", "u1"), ("bt", "u1"), ("pt", "u1"),
                      ("mono", "u1"), ("x", "<f8", 3), ("v", "<f8", 3), ("f", "<f8", 3)])
    rec = np.frombuffer(mv, dtype, n, p)
    return World(box=box, dt=dt, lam=lam, seed=seed, t=t, conservative=cons, dissipative=diss,
                 stationary=stationary, polymer_types=pts, poly_type=poly_type,
                 poly_start=poly_start, poly_beads=poly_beads,
                 polymer_id=rec["pid"].copy(), polymer_offset=rec["off"].copy(),
                 bead_type=rec["bt"].copy(), polymer_type_of_bead=rec["pt"].copy(),
                 is_monomer=rec["mono"].astype(bool), x=rec["x"].copy(), v=rec["v"].copy(),
                 f=rec["f"].copy())
