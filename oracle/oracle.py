"""ctypes binding of the oracle (TEST INFRASTRUCTURE ONLY).

The oracle is a C restatement of the reference's FP64 half-step engine (pdpd_oracle.c).
Only tests/, the smoke check and bench.py's CPU-baseline and reference arms use it, as the
checker or as the timed CPU implementation; the GPU engine never does.
"""

from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None


class _World(C.Structure):
    _fields_ = [
        ("box", C.c_int32 * 3), ("dt", C.c_double), ("lam", C.c_double),
        ("seed", C.c_uint64), ("t", C.c_int64), ("n_types", C.c_uint32),
        ("conservative", C.c_void_p), ("dissipative", C.c_void_p),
        ("n_beads", C.c_uint32), ("hash", C.c_void_p),
        ("x", C.c_void_p), ("v", C.c_void_p), ("f", C.c_void_p),
        ("n_bonds", C.c_uint32), ("bond_beads", C.c_void_p), ("bond_kappa", C.c_void_p),
        ("bond_r0", C.c_void_p), ("n_angles", C.c_uint32), ("angle_beads", C.c_void_p),
        ("angle_kappa", C.c_void_p), ("angle_theta0", C.c_void_p), ("stationary", C.c_uint32),
        ("cell_conservative", C.c_void_p), ("cell_dissipative", C.c_void_p),
    ]


class _Obs(C.Structure):
    _fields_ = [("ke2", C.c_double), ("virial", C.c_double), ("momentum", C.c_double * 3)]


def build():
    """Compile liboracle.so with the committed Makefile (gcc, -ffp-contract=off)."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(_HERE, "liboracle.so")
        if not os.path.exists(path):
            build()
        L = C.CDLL(path)
        L.pdo_mix64_m2.restype = C.c_uint64
        L.pdo_mix64_m2.argtypes = [C.c_uint64]
        L.pdo_t_hash.restype = C.c_uint64
        L.pdo_t_hash.argtypes = [C.c_uint32, C.c_uint64]
        L.pdo_hash_rng_sym.restype = C.c_uint32
        L.pdo_hash_rng_sym.argtypes = [C.c_uint64, C.c_uint32, C.c_uint32]
        L.pdo_default_hash.restype = C.c_float
        L.pdo_default_hash.argtypes = [C.c_uint64, C.c_uint32, C.c_uint32]
        L.pdo_hash_batch.restype = None
        L.pdo_hash_batch.argtypes = [C.c_size_t] + [C.c_void_p] * 7
        L.pdo_run.restype = C.c_int
        L.pdo_run.argtypes = [C.POINTER(_World), C.c_uint32, C.c_int, C.c_char_p, C.c_size_t]
        L.pdo_cell_index.restype = None
        L.pdo_cell_index.argtypes = [C.POINTER(_World), C.c_void_p]
        L.pdo_observe.restype = None
        L.pdo_observe.argtypes = [C.POINTER(_World), C.c_int, C.POINTER(_Obs), C.c_uint32,
                                  C.c_void_p, C.c_uint32, C.c_void_p]
        _LIB = L
    return _LIB


def _ptr(a):
    return a.ctypes.data if a is not None and a.size else None


class OracleWorld:
    """Owns contiguous copies of a :class:`pdpd_world.World` and steps them with the oracle."""

    def __init__(self, world):
        self.world = world
        self.box = np.asarray(world.box, np.int32)
        self.cons = np.ascontiguousarray(world.conservative, np.float64)
        self.diss = np.ascontiguousarray(world.dissipative, np.float64)
        self.hash = np.ascontiguousarray(world.hashes(), np.uint32)
        self.x = np.ascontiguousarray(world.x, np.float64).copy()
        self.v = np.ascontiguousarray(world.v, np.float64).copy()
        self.f = np.ascontiguousarray(world.f, np.float64).copy()
        bb, bk, br, ab, ak, at = world.flat_bonds()
        self.bb, self.bk, self.br = (np.ascontiguousarray(bb, np.uint32),
                                     np.ascontiguousarray(bk), np.ascontiguousarray(br))
        self.ab, self.ak, self.at = (np.ascontiguousarray(ab, np.uint32),
                                     np.ascontiguousarray(ak), np.ascontiguousarray(at))
        self.t = int(world.t)
        self.stationary = sum(1 << k for k, st in enumerate(np.asarray(world.stationary, bool)) if st)
        cc = getattr(world, "cell_conservative", None)
        cd = getattr(world, "cell_dissipative", None)
        self.cell_a = None if cc is None else np.ascontiguousarray(cc, np.float64)
        self.cell_g = None if cd is None else np.ascontiguousarray(cd, np.float64)

    def _struct(self):
        s = _World()
        for i in range(3):
            s.box[i] = int(self.box[i])
        s.dt, s.lam = float(self.world.dt), float(self.world.lam)
        s.seed, s.t = int(self.world.seed) & 0xFFFFFFFFFFFFFFFF, int(self.t)
        s.n_types = self.cons.shape[0]
        s.conservative, s.dissipative = _ptr(self.cons), _ptr(self.diss)
        s.n_beads = self.x.shape[0]
        s.hash, s.x, s.v, s.f = _ptr(self.hash), _ptr(self.x), _ptr(self.v), _ptr(self.f)
        s.n_bonds = self.bb.shape[0]
        s.bond_beads, s.bond_kappa, s.bond_r0 = _ptr(self.bb), _ptr(self.bk), _ptr(self.br)
        s.n_angles = self.ab.shape[0]
        s.angle_beads, s.angle_kappa, s.angle_theta0 = _ptr(self.ab), _ptr(self.ak), _ptr(self.at)
        s.stationary = self.stationary
        s.cell_conservative = None if self.cell_a is None else _ptr(self.cell_a)
        s.cell_dissipative = None if self.cell_g is None else _ptr(self.cell_g)
        return s

    def run(self, nsteps, nthreads=1):
        s = self._struct()
        err = C.create_string_buffer(256)
        rc = lib().pdo_run(C.byref(s), nsteps, nthreads, err, 256)
        self.t = s.t
        if rc != 0:
            raise RuntimeError("oracle: " + err.value.decode())
        return self

    def cell_index(self):
        s = self._struct()
        out = np.zeros(self.x.shape[0], np.uint32)
        lib().pdo_cell_index(C.byref(s), _ptr(out))
        return out

    def observe(self, n_bins=50, n_bond_bins=100, nthreads=1):
        s = self._struct()
        obs = _Obs()
        nt = self.cons.shape[0]
        rdf = np.zeros(nt * nt * n_bins, np.uint64)
        bh = np.zeros(n_bond_bins, np.uint64)
        lib().pdo_observe(C.byref(s), nthreads, C.byref(obs), n_bins, _ptr(rdf), n_bond_bins,
                          _ptr(bh))
        return {"ke2": obs.ke2, "virial": obs.virial, "momentum": np.array(obs.momentum[:]),
                "rdf": rdf.reshape(nt, nt, n_bins), "bond_hist": bh}


def hash_batch(t, seed, a, b):
    t = np.ascontiguousarray(t, np.uint32)
    seed = np.ascontiguousarray(seed, np.uint64)
    a = np.ascontiguousarray(a, np.uint32)
    b = np.ascontiguousarray(b, np.uint32)
    n = t.size
    th = np.zeros(n, np.uint64)
    h = np.zeros(n, np.uint32)
    u = np.zeros(n, np.float32)
    lib().pdo_hash_batch(n, _ptr(t), _ptr(seed), _ptr(a), _ptr(b), _ptr(th), _ptr(h), _ptr(u))
    return th, h, u
