"""Python mirror of the reference's ``DPDEngine`` plug-in interface over the engine's C ABI.

``GB300DPDEngine`` has the members of ``class DPDEngine`` (reference
include/dpd/core/dpd_engine.hpp:10-216) with the same meaning:

=========================  ==============================================================
``CanSupport(world)``      "" if the world can be attached, else the reason (:57-128)
``Attach(world)``          copy the world to the GPU; ``Attach(None)`` detaches (:177)
``Run(n)``                 advance n steps; the world's x/v/f/t are updated on return (:185)
``Run(count, size, cb)``   interval runs with a callback; returns steps done (:195-215)
``GetMaxBondLength()``     2.0 (:130)
``GetTimings()``           dict of ``timings_t`` fields (:38-46, :145-148)
``GetConfigEntries()``     list of (name, description, value) (:160-164)
``SetConfigEntry(k, v)``   raises on an unknown key (:166-169)
=========================  ==============================================================

Errors are raised as ``RuntimeError`` (the reference throws ``std::runtime_error``).  The
shared library must exist (built by ``build.py``); there is no CPU fallback.
"""

from __future__ import annotations

import copy
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libpdpd_gb300.so")

PDPD_FP32, PDPD_FP64 = 0, 1
# PDPD_NOALLOC_MAX_BEADS / PDPD_NOALLOC_MAX_CELLS: the fixed scratch size of pdpd_step_noalloc.
NOALLOC_MAX_BEADS, NOALLOC_MAX_CELLS = 65536, 32768
STATUS = {0: "PDPD_OK", 1: "PDPD_E_INVALID", 2: "PDPD_E_UNSUPPORTED", 3: "PDPD_E_CUDA",
          4: "PDPD_E_STATE", 5: "PDPD_E_BOND_SNAPPED", 6: "PDPD_E_BEAD_LOST", 7: "PDPD_E_NOMEM"}

# Every symbol include/pdpd_gpu.h declares.
EXPORTED = ["pdpd_create", "pdpd_destroy", "pdpd_last_error", "pdpd_can_support",
            "pdpd_max_bond_length", "pdpd_attach", "pdpd_attach_batch", "pdpd_run",
            "pdpd_run_async", "pdpd_sync", "pdpd_stream", "pdpd_read_state", "pdpd_read_states",
            "pdpd_run_intervals", "pdpd_get_timings", "pdpd_get_config", "pdpd_set_config",
            "pdpd_kernel_launches", "pdpd_rng_eval", "pdpd_profile_run", "pdpd_step_noalloc",
            "pdpd_observe", "pdpd_log_pair_terms", "pdpd_v2binary_prepare", "pdpd_v2binary_encode",
            "pdpd_v2binary_decode", "pdpd_server_create", "pdpd_server_submit", "pdpd_server_drain",
            "pdpd_server_config", "pdpd_server_stats_get", "pdpd_server_engine",
            "pdpd_server_destroy"]


class PdpdWorld(C.Structure):
    _fields_ = [
        ("box", C.c_int32 * 3), ("dt", C.c_double), ("lam", C.c_double), ("seed", C.c_uint64),
        ("t", C.c_int64), ("n_bead_types", C.c_uint32), ("conservative", C.c_void_p),
        ("dissipative", C.c_void_p), ("stationary", C.c_void_p), ("n_beads", C.c_uint32),
        ("hash", C.c_void_p), ("x", C.c_void_p), ("v", C.c_void_p), ("f", C.c_void_p),
        ("bead_stride_bytes", C.c_size_t), ("n_bonds", C.c_uint32), ("bond_beads", C.c_void_p),
        ("bond_kappa", C.c_void_p), ("bond_r0", C.c_void_p), ("n_angles", C.c_uint32),
        ("angle_beads", C.c_void_p), ("angle_kappa", C.c_void_p), ("angle_theta0", C.c_void_p),
        ("cell_conservative", C.c_void_p), ("cell_dissipative", C.c_void_p),
    ]


class PdpdStateView(C.Structure):
    _fields_ = [("x", C.c_void_p), ("v", C.c_void_p), ("f", C.c_void_p), ("t", C.c_void_p)]


class PdpdTimings(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("compile", "aquire", "configure",
                                          "execute_to_first_bead", "execute_to_last_bead",
                                          "perf_counters")]


class PdpdPhaseTimes(C.Structure):
    _fields_ = [("force_ms", C.c_double), ("sort_ms", C.c_double), ("other_ms", C.c_double),
                ("force_launches", C.c_uint32), ("sort_launches", C.c_uint32)]


# pdpd_pair_terms (include/pdpd_gpu.h): one pair of the per-pair force log.
PAIR_TERMS_DTYPE = np.dtype([("t", "<i8"), ("home_id", "<u4"), ("other_id", "<u4"),
                             ("home_hash", "<u4"), ("other_hash", "<u4"), ("dx", "<f8", 3),
                             ("dr", "<f8"), ("inv_root_dt", "<f8"), ("gammap", "<f8"), ("rng", "<f8"),
                             ("con", "<f8"), ("diss", "<f8"), ("rng_scale", "<f8"), ("rand", "<f8"),
                             ("f", "<f8", 3)])

# The names the reference's calc_force logs a pair's terms under
# (dpd_maths_core_half_step.hpp:134-148), with the record fields that hold them.
PAIR_LOG_PROPERTIES = [("dx", "dx"), ("dr", "dr"), ("dpd-invrootdt", "inv_root_dt"),
                       ("dpd-gammap", "gammap"), ("dpd-rng", "rng"), ("dpd-con", "con"),
                       ("dpd-diss", "diss"), ("dpd-rng-scale", "rng_scale"), ("dpd-rand", "rand"),
                       ("f_next_dpd", "f")]


def _log_value(v):
    """A value as the reference's FileLogger prints it (logging_impl.hpp:27-34): an integer in
    [0, 2^32) as an integer, anything else as an ostream prints a double (%g, 6 digits)."""
    v = float(v)
    if v == round(v) and 0 <= v < 2.0 ** 32:
        return str(int(v))
    return "%g" % v


def force_log_lines(records, prefix=""):
    """The pair records in the reference's FileLogger text format (logging_impl.hpp:75-86):
    'Prop,t,home,other,,name,v0,v1,v2' with reduced hashes (hash & 0x0fffffff), one line per
    property, in the reference's property order -- to diff against a reference log."""
    lines = []
    for r in records:
        h0, h1 = int(r["home_hash"]) & 0x0FFFFFFF, int(r["other_hash"]) & 0x0FFFFFFF
        for name, field in PAIR_LOG_PROPERTIES:
            vals = np.atleast_1d(r[field])
            cells = [_log_value(x) for x in vals] + [""] * (3 - vals.size)
            lines.append(f"{prefix}Prop,{int(r['t'])},{h0},{h1},,{name}," + ",".join(cells))
    return lines


class PdpdObservables(C.Structure):
    _fields_ = [("ke2", C.c_double), ("momentum", C.c_double * 3), ("virial", C.c_double)]


class PdpdServerStats(C.Structure):
    _fields_ = [("jobs_submitted", C.c_uint64), ("jobs_done", C.c_uint64),
                ("jobs_failed", C.c_uint64), ("bead_steps", C.c_uint64), ("repacks", C.c_uint64),
                ("max_active", C.c_uint32), ("pad", C.c_uint32), ("busy_s", C.c_double),
                ("wall_s", C.c_double), ("latency_p50_s", C.c_double),
                ("latency_p99_s", C.c_double), ("latency_max_s", C.c_double),
                ("repack_s", C.c_double), ("wasted_bead_steps", C.c_uint64),
                ("step_s", C.c_double), ("host_gap_s", C.c_double), ("callback_s", C.c_double),
                ("epochs", C.c_uint64), ("between_s", C.c_double), ("copy_wait_s", C.c_double),
                ("sync_wait_s", C.c_double), ("snap_alloc_s", C.c_double),
                ("post_launch_s", C.c_double)]


INTERVAL_FN = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_int64)
JOB_FN = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_uint64, C.c_int64, C.POINTER(C.c_double),
                     C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_size_t, C.c_uint32, C.c_int)

_LIB = None


def lib():
    """Load libpdpd_gb300.so.  Raises if it has not been built: the engine has no fallback."""
    global _LIB
    if _LIB is not None:
        return _LIB
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"{LIB_PATH} is missing: run build.py (or __graft_entry__.build())")
    L = C.CDLL(LIB_PATH)
    vp, u32, i32 = C.c_void_p, C.c_uint32, C.c_int
    sig = {
        "pdpd_create": (i32, [i32, i32, C.POINTER(vp)]),
        "pdpd_destroy": (None, [vp]),
        "pdpd_last_error": (C.c_char_p, [vp]),
        "pdpd_can_support": (i32, [C.POINTER(PdpdWorld), C.c_char_p, C.c_size_t]),
        "pdpd_max_bond_length": (C.c_double, []),
        "pdpd_attach": (i32, [vp, C.POINTER(PdpdWorld)]),
        "pdpd_attach_batch": (i32, [vp, C.POINTER(PdpdWorld), u32]),
        "pdpd_run": (i32, [vp, u32]),
        "pdpd_run_async": (i32, [vp, u32]),
        "pdpd_sync": (i32, [vp]),
        "pdpd_stream": (vp, [vp]),
        "pdpd_read_state": (i32, [vp, u32, vp, vp, vp, C.c_size_t, C.POINTER(C.c_int64)]),
        "pdpd_read_states": (i32, [vp, u32, C.POINTER(PdpdStateView), C.c_size_t]),
        "pdpd_run_intervals": (i32, [vp, C.c_int32, u32, vp, vp, vp, C.c_size_t, INTERVAL_FN, vp,
                                     C.POINTER(u32)]),
        "pdpd_get_timings": (i32, [vp, C.POINTER(PdpdTimings)]),
        "pdpd_get_config": (i32, [vp, u32, C.c_char_p, C.c_size_t, C.c_char_p, C.c_size_t,
                                  C.c_char_p, C.c_size_t]),
        "pdpd_set_config": (i32, [vp, C.c_char_p, C.c_char_p]),
        "pdpd_kernel_launches": (C.c_uint64, [vp]),
        "pdpd_rng_eval": (i32, [C.c_size_t, vp, vp, vp, vp, vp, vp]),
        "pdpd_profile_run": (i32, [vp, u32, C.POINTER(PdpdPhaseTimes)]),
        "pdpd_step_noalloc": (i32, [C.POINTER(PdpdWorld), vp, vp, vp, vp, u32, vp]),
        "pdpd_observe": (i32, [vp, u32, C.POINTER(PdpdObservables), u32, vp, u32, vp]),
        "pdpd_log_pair_terms": (i32, [vp, u32, vp, u32, vp, u32, C.POINTER(u32)]),
        "pdpd_v2binary_prepare": (i32, [vp, u32, u32, vp, vp, vp, vp, C.POINTER(C.c_size_t)]),
        "pdpd_v2binary_encode": (i32, [vp, u32, vp, C.c_size_t, C.POINTER(C.c_size_t)]),
        "pdpd_v2binary_decode": (i32, [vp, u32, vp, C.c_size_t]),
        "pdpd_server_create": (i32, [i32, i32, C.c_size_t, u32, C.POINTER(vp)]),
        "pdpd_server_submit": (i32, [vp, C.POINTER(PdpdWorld), u32, JOB_FN, vp,
                                     C.POINTER(C.c_uint64)]),
        "pdpd_server_drain": (i32, [vp]),
        "pdpd_server_config": (i32, [vp, C.c_char_p, C.c_char_p]),
        "pdpd_server_stats_get": (i32, [vp, C.POINTER(PdpdServerStats)]),
        "pdpd_server_engine": (vp, [vp]),
        "pdpd_server_destroy": (None, [vp]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _LIB = L
    return L


def _p(a):
    """Address of an array's first element (None for a missing or empty array): through the
    buffer protocol where the array is writable (a third of the cost of ``a.ctypes``, which
    counts at one call per array of every world of a batch), else ``a.ctypes``."""
    if a is None or not a.size:
        return None
    try:
        return C.addressof(C.c_char.from_buffer(a))
    except (TypeError, ValueError, BufferError):
        return a.ctypes.data


def _dest(world, name, n):
    """Where a read-back of a World's x, v or f goes: its own array when that is a writable,
    C-contiguous float64 (n, 3) array -- written in place, as the reference's engines write
    the WorldState's beads (its pages are already mapped, unlike a new array's) -- else a new
    array."""
    a = getattr(world, name, None) if world is not None else None
    if isinstance(a, np.ndarray) and a.dtype == np.float64 and a.shape == (n, 3):
        fl = a.flags
        if fl.c_contiguous and fl.writeable:
            return a
    return np.empty((n, 3))


class _Flat:
    """Contiguous arrays of one World in the C ABI's layout, kept alive with the struct.  The
    topology part (bead hashes, flat bond lists: read-only arrays a World computes once) is
    laid into a struct template kept with the World and shared by its copies; each call fills
    in the state and parameters."""

    def __init__(self, world):
        tmpl, self.topo = _topology_struct(world)
        self.cons = np.ascontiguousarray(world.conservative, np.float64)
        self.diss = np.ascontiguousarray(world.dissipative, np.float64)
        self.stat = np.ascontiguousarray(world.stationary, np.uint8)
        self.x = np.ascontiguousarray(world.x, np.float64)
        self.v = np.ascontiguousarray(world.v, np.float64)
        self.f = np.ascontiguousarray(world.f, np.float64)
        s = PdpdWorld.from_buffer_copy(tmpl)
        s.box[0], s.box[1], s.box[2] = int(world.box[0]), int(world.box[1]), int(world.box[2])
        s.dt, s.lam = float(world.dt), float(world.lam)
        s.seed, s.t = int(world.seed) & 0xFFFFFFFFFFFFFFFF, int(world.t)
        s.n_bead_types = self.cons.shape[0]
        s.conservative, s.dissipative, s.stationary = _p(self.cons), _p(self.diss), _p(self.stat)
        s.n_beads = self.x.shape[0]
        s.x, s.v, s.f = _p(self.x), _p(self.v), _p(self.f)
        cc, cd = getattr(world, "cell_conservative", None), getattr(world, "cell_dissipative", None)
        self.cell_a = None if cc is None else np.ascontiguousarray(cc, np.float64)
        self.cell_g = None if cd is None else np.ascontiguousarray(cd, np.float64)
        s.cell_conservative = None if self.cell_a is None else self.cell_a.ctypes.data
        s.cell_dissipative = None if self.cell_g is None else self.cell_g.ctypes.data
        self.struct = s


_TOPOLOGY_ARRAYS = ("bead_type", "is_monomer", "polymer_id", "polymer_offset", "poly_type", "poly_start",
                    "poly_beads")


def _topology_struct(world):
    """A PdpdWorld with the hash and bond fields of the World's topology set (and the arrays
    they point to), cached with the World (and its copies) while its topology arrays are the
    same objects and its polymer types equal those the struct was made from -- what the
    World's own hash and bond-list caches depend on."""
    cache = world.__dict__.setdefault("_cache", {})
    hit = cache.get("abi")
    if hit is not None:
        d = world.__dict__
        if all(d.get(k) is a for k, a in zip(_TOPOLOGY_ARRAYS, hit[4])) and hit[5] == world.polymer_types:
            return hit[2], hit[3]
    hash_ = world.hashes()
    bonds = world.flat_bonds()
    h = np.ascontiguousarray(hash_, np.uint32)
    bb, bk, br, ab, ak, at = bonds
    arrs = (h, np.ascontiguousarray(bb, np.uint32), np.ascontiguousarray(bk), np.ascontiguousarray(br),
            np.ascontiguousarray(ab, np.uint32), np.ascontiguousarray(ak), np.ascontiguousarray(at))
    s = PdpdWorld()
    s.hash = _p(arrs[0])
    s.bead_stride_bytes = 24
    s.n_bonds, s.bond_beads, s.bond_kappa, s.bond_r0 = arrs[1].shape[0], _p(arrs[1]), _p(arrs[2]), _p(arrs[3])
    s.n_angles, s.angle_beads, s.angle_kappa, s.angle_theta0 = (arrs[4].shape[0], _p(arrs[4]), _p(arrs[5]),
                                                                _p(arrs[6]))
    cache["abi"] = (hash_, bonds, s, arrs, tuple(getattr(world, k) for k in _TOPOLOGY_ARRAYS),
                    copy.deepcopy(world.polymer_types), bytes(s))
    return s, arrs


_WORLD_DTYPE = np.dtype(PdpdWorld)
_VIEW_DTYPE = np.dtype(PdpdStateView)


def _flat_batch(worlds):
    """The PdpdWorld array of a batch attach, byte for byte the structs ``_Flat`` makes, built
    column by column: each World's topology part as the bytes cached with it, its state and
    parameters gathered into lists and written per field (the per-World cost of building
    ctypes structs one by one counts once per state of a large batch).  Returns the array
    and the arrays it points to, to keep alive for the call."""
    n = len(worlds)
    topo, keep = [], []
    box = np.empty((n, 3), np.int32)
    dt, lam, seed, t = [], [], [], []
    ntypes, nbeads = [], []
    ptr = {k: [] for k in ("conservative", "dissipative", "stationary", "x", "v", "f",
                           "cell_conservative", "cell_dissipative")}
    for i, w in enumerate(worlds):
        _topology_struct(w)
        topo.append(w.__dict__["_cache"]["abi"][6])
        cons = np.ascontiguousarray(w.conservative, np.float64)
        diss = np.ascontiguousarray(w.dissipative, np.float64)
        stat = w.stationary
        stat = (stat.view(np.uint8) if isinstance(stat, np.ndarray) and stat.dtype == np.bool_
                and stat.flags.c_contiguous else np.ascontiguousarray(stat, np.uint8))
        x = np.ascontiguousarray(w.x, np.float64)
        v = np.ascontiguousarray(w.v, np.float64)
        f = np.ascontiguousarray(w.f, np.float64)
        cc, cd = getattr(w, "cell_conservative", None), getattr(w, "cell_dissipative", None)
        cc = None if cc is None else np.ascontiguousarray(cc, np.float64)
        cd = None if cd is None else np.ascontiguousarray(cd, np.float64)
        keep.append((cons, diss, stat, x, v, f, cc, cd))
        box[i] = w.box
        dt.append(float(w.dt))
        lam.append(float(w.lam))
        seed.append(int(w.seed) & 0xFFFFFFFFFFFFFFFF)
        t.append(int(w.t))
        ntypes.append(cons.shape[0])
        nbeads.append(x.shape[0])
        for k, a in zip(ptr, (cons, diss, stat, x, v, f, cc, cd)):
            ptr[k].append(_p(a) or 0)
    out = np.frombuffer(b"".join(topo), _WORLD_DTYPE).copy() if n else np.zeros(0, _WORLD_DTYPE)
    out["box"] = box
    out["dt"], out["lam"] = dt, lam
    out["seed"] = np.array(seed, np.uint64)
    out["t"] = t
    out["n_bead_types"], out["n_beads"] = ntypes, nbeads
    for k, v in ptr.items():
        out[k] = np.array(v, np.uint64)
    return out, keep


def can_support(world) -> str:
    """``DPDEngine::CanSupport``: empty string when the world can run on this engine."""
    fl = _Flat(world)
    buf = C.create_string_buffer(512)
    rc = lib().pdpd_can_support(C.byref(fl.struct), buf, 512)
    return "" if rc == 0 else buf.value.decode()


def rng_eval(t, seed, a, b):
    """The device RNG (hash_rng_sym and default_hash) on arrays; returns (h, u)."""
    t = np.ascontiguousarray(t, np.uint32)
    seed = np.ascontiguousarray(seed, np.uint64)
    a = np.ascontiguousarray(a, np.uint32)
    b = np.ascontiguousarray(b, np.uint32)
    h = np.zeros(t.size, np.uint32)
    u = np.zeros(t.size, np.float32)
    rc = lib().pdpd_rng_eval(t.size, _p(t), _p(seed), _p(a), _p(b), _p(h), _p(u))
    if rc != 0:
        raise RuntimeError(f"pdpd_rng_eval: {STATUS.get(rc)}: {lib().pdpd_last_error(None).decode()}")
    return h, u


def step_noalloc(world, d_x, d_v, d_f, d_hash, n_steps, t=None, stream=None):
    """``pdpd_step_noalloc``: advance a bond-free world by n_steps (FP64) on device arrays
    the caller owns (integer device addresses: x, v, f with 3 doubles per bead, hash with one
    uint32 per bead), without the library allocating any memory.  ``t`` is the time of the
    state in the arrays (default ``world.t``)."""
    fl = _Flat(world)
    if t is not None:
        fl.struct.t = int(t)
    rc = lib().pdpd_step_noalloc(C.byref(fl.struct), d_x, d_v, d_f, d_hash, int(n_steps), stream)
    if rc != 0:
        raise RuntimeError(f"pdpd_step_noalloc: {STATUS.get(rc)}: {lib().pdpd_last_error(None).decode()}")


class GB300DPDEngine:
    """A GPU DPD engine.  ``precision`` is ``"fp32"`` or ``"fp64"``."""

    def __init__(self, precision="fp32", device=-1):
        self.precision = precision
        code = {"fp32": PDPD_FP32, "fp64": PDPD_FP64}[precision]
        h = C.c_void_p()
        rc = lib().pdpd_create(code, device, C.byref(h))
        if rc != 0:
            raise RuntimeError(f"pdpd_create: {STATUS.get(rc)}: {lib().pdpd_last_error(None).decode()}")
        self._h = h
        self._worlds = []

    # -- life-cycle ---------------------------------------------------------------------
    def close(self):
        if getattr(self, "_h", None):
            lib().pdpd_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc, what):
        if rc != 0:
            msg = lib().pdpd_last_error(self._h).decode()
            raise RuntimeError(f"{what}: {STATUS.get(rc, rc)}: {msg}")

    # -- DPDEngine interface -----------------------------------------------------------
    def CanSupport(self, world) -> str:
        return can_support(world)

    def GetMaxBondLength(self) -> float:
        return lib().pdpd_max_bond_length()

    def Attach(self, world):
        if world is None:
            self._check(lib().pdpd_attach(self._h, None), "Attach")
            self._worlds = []
            return
        fl = _Flat(world)
        self._check(lib().pdpd_attach(self._h, C.byref(fl.struct)), "Attach")
        self._worlds = [world]

    def AttachBatch(self, worlds):
        arr, keep = _flat_batch(worlds)
        self._check(lib().pdpd_attach_batch(self._h, arr.ctypes.data_as(C.POINTER(PdpdWorld)), len(arr)),
                    "AttachBatch")
        del keep
        self._worlds = list(worlds)

    def Run(self, *args):
        if len(args) == 1:
            self._check(lib().pdpd_run(self._h, int(args[0])), "Run")
            if len(self._worlds) == 1:
                self.read_state(0, into=self._worlds[0])
            elif self._worlds:
                self.read_states(into=self._worlds)
            return None
        count, size, cb = args
        return self._run_intervals(int(count), int(size), cb)

    def _run_intervals(self, count, size, cb):
        if len(self._worlds) != 1:
            raise RuntimeError("interval runs need exactly one attached world")
        w = self._worlds[0]
        x = np.ascontiguousarray(w.x)
        v = np.ascontiguousarray(w.v)
        f = np.ascontiguousarray(w.f)
        w.x, w.v, w.f = x, v, f
        err = []

        def tramp(_user, t):
            try:
                w.t = int(t)
                return 1 if cb() else 0
            except BaseException as e:  # stop the run, re-raise below
                err.append(e)
                return 0

        fn = INTERVAL_FN(tramp)
        done = C.c_uint32(0)
        rc = lib().pdpd_run_intervals(self._h, count, size, _p(x), _p(v), _p(f), 24, fn, None,
                                      C.byref(done))
        if err:
            raise err[0]
        self._check(rc, "Run(intervals)")
        return int(done.value)

    def GetTimings(self):
        t = PdpdTimings()
        self._check(lib().pdpd_get_timings(self._h, C.byref(t)), "GetTimings")
        return {n: getattr(t, n) for n, _ in PdpdTimings._fields_}

    def GetConfigEntries(self):
        out = []
        i = 0
        while True:
            n, d, v = (C.create_string_buffer(128) for _ in range(3))
            if lib().pdpd_get_config(self._h, i, n, 128, d, 128, v, 128) != 0:
                break
            out.append((n.value.decode(), d.value.decode(), v.value.decode()))
            i += 1
        return out

    def SetConfigEntry(self, key, value):
        self._check(lib().pdpd_set_config(self._h, key.encode(), str(value).encode()),
                    "SetConfigEntry")

    # -- extras -----------------------------------------------------------------------
    def run_async(self, n):
        self._check(lib().pdpd_run_async(self._h, int(n)), "run_async")

    def sync(self):
        self._check(lib().pdpd_sync(self._h), "sync")

    def stream(self):
        return lib().pdpd_stream(self._h)

    def profile_run(self, n):
        """Run n steps launching kernels one by one with CUDA events between phases; returns
        per-phase device milliseconds (the trajectory equals Run(n)'s)."""
        pt = PdpdPhaseTimes()
        self._check(lib().pdpd_profile_run(self._h, int(n), C.byref(pt)), "profile_run")
        return {n_: getattr(pt, n_) for n_, _ in PdpdPhaseTimes._fields_}

    def observe(self, world_index=0, n_bins=50, n_bond_bins=100):
        """FP64 GPU reductions of the current state of one world: ke2 (sum |v|^2), momentum,
        virial (conservative pairs + Hookean bonds), per-type-pair RDF counts over r in [0,1)
        and the Hookean bond-length histogram over [0, 2)."""
        nt = self._worlds[world_index].n_types
        rdf = np.zeros(nt * nt * n_bins, np.uint64)
        bh = np.zeros(n_bond_bins, np.uint64)
        o = PdpdObservables()
        self._check(lib().pdpd_observe(self._h, world_index, C.byref(o), n_bins, _p(rdf),
                                       n_bond_bins, _p(bh)), "observe")
        return {"ke2": o.ke2, "virial": o.virial, "momentum": np.array(o.momentum[:]),
                "rdf": rdf.reshape(nt, nt, n_bins), "bond_hist": bh}

    def log_pair_terms(self, bead_ids, world_index=0, per_bead_capacity=256):
        """Advance one step (as Run(1)) and return the pair terms of that step for the given
        beads of world ``world_index``: a structured array (PAIR_TERMS_DTYPE, the C ABI's
        pdpd_pair_terms) grouped by bead in ascending id order, each bead's pairs in the
        reference's walk order -- what the reference's ForceLogging logs from calc_force.
        Room is made for per_bead_capacity pairs per bead (density 3 gives ~13); a step with
        more raises, and its records are lost (the step itself has run)."""
        ids = np.ascontiguousarray(np.unique(np.asarray(bead_ids, np.int64)).astype(np.uint32))
        cap = max(1, per_bead_capacity * ids.size)
        out = np.zeros(cap, PAIR_TERMS_DTYPE)
        n = C.c_uint32(0)
        self._check(lib().pdpd_log_pair_terms(self._h, world_index, _p(ids), ids.size, _p(out), cap,
                                              C.byref(n)), "log_pair_terms")
        if n.value > cap:
            raise RuntimeError(f"log_pair_terms: {n.value} pairs, room for {cap}")
        return out[:n.value]

    def kernel_launches(self):
        return int(lib().pdpd_kernel_launches(self._h))

    # -- v2binary snapshots ---------------------------------------------------------------
    def v2binary_prepare(self, world_index=0, polymer_ids=None) -> int:
        """Lay out the v2binary section of attached world ``world_index`` from its polymers
        (the World's ``poly_type`` / ``poly_start`` / ``poly_beads``); returns its size."""
        w = self._worlds[world_index]
        pt = np.ascontiguousarray(w.poly_type, np.uint32)
        ps = np.ascontiguousarray(w.poly_start, np.uint32)
        pb = np.ascontiguousarray(w.poly_beads, np.uint32)
        pid = None if polymer_ids is None else np.ascontiguousarray(polymer_ids, np.uint32)
        size = C.c_size_t(0)
        self._check(lib().pdpd_v2binary_prepare(self._h, world_index, len(pt), _p(pid), _p(pt),
                                                _p(ps), _p(pb), C.byref(size)), "v2binary_prepare")
        return int(size.value)

    def v2binary_encode(self, world_index=0) -> np.ndarray:
        """The BinaryData section of the world's current state, encoded on the GPU (uint8
        array; ``.tobytes()`` for bytes)."""
        size = C.c_size_t(0)
        self._check(lib().pdpd_v2binary_encode(self._h, world_index, None, 0, C.byref(size)),
                    "v2binary_encode")
        out = np.empty(max(1, size.value), np.uint8)
        self._check(lib().pdpd_v2binary_encode(self._h, world_index, out.ctypes.data, out.size,
                                               C.byref(size)), "v2binary_encode")
        return out[:size.value]

    def v2binary_decode(self, section, world_index=0):
        """Set the world's x, v, f from a BinaryData section (bytes or uint8 array), decoded
        on the GPU."""
        buf = np.ascontiguousarray(np.frombuffer(section, np.uint8))
        self._check(lib().pdpd_v2binary_decode(self._h, world_index, buf.ctypes.data if buf.size else None,
                                               buf.size), "v2binary_decode")
        if self._worlds:
            self.read_state(world_index, into=self._worlds[world_index])

    def read_states(self, into=None):
        """Every attached world's x, v, f, t at once (one device unsort and copy); returns a
        list of (x, v, f, t), and writes them into the given Worlds when ``into`` is given."""
        n = len(self._worlds)
        dst = into if into is not None else [None] * n
        arrs = [(_dest(d, "x", w.n_beads), _dest(d, "v", w.n_beads), _dest(d, "f", w.n_beads))
                for w, d in zip(self._worlds, dst)]
        ts = np.zeros(max(1, n), np.int64)
        views = np.zeros(max(1, n), _VIEW_DTYPE)  # (filled per field: one World costs little)
        for q, k in enumerate(("x", "v", "f")):
            views[k][:n] = [_p(a[q]) or 0 for a in arrs]
        views["t"] = ts.ctypes.data + 8 * np.arange(max(1, n), dtype=np.uint64)
        self._check(lib().pdpd_read_states(self._h, n, views.ctypes.data_as(C.POINTER(PdpdStateView)), 24),
                    "read_states")
        out = [(x, v, f, int(ts[i])) for i, (x, v, f) in enumerate(arrs)]
        if into is not None:
            for w, (x, v, f, t) in zip(into, out):
                if w.x is not x or w.v is not v or w.f is not f:  # (else written in place)
                    w.x, w.v, w.f = x, v, f
                w.t = t
        return out

    def read_state(self, world_index=0, into=None):
        """Copy world ``world_index``'s x, v, f, t to numpy (into a World when given)."""
        n = (self._worlds[world_index].n_beads if self._worlds else 0)
        x, v, f = (_dest(into, k, n) for k in ("x", "v", "f"))
        t = C.c_int64(0)
        self._check(lib().pdpd_read_state(self._h, world_index, _p(x), _p(v), _p(f), 24,
                                          C.byref(t)), "read_state")
        if into is not None:
            into.x, into.v, into.f, into.t = x, v, f, int(t.value)
        return x, v, f, int(t.value)


def _rows(ptr, n, stride_bytes):
    """Copy n vectors of 3 doubles, stride_bytes apart, out of a callback's pointer."""
    if n == 0:
        return np.empty((0, 3))
    step = stride_bytes // 8
    flat = np.ctypeslib.as_array(ptr, shape=((n - 1) * step + 3,))
    return np.lib.stride_tricks.as_strided(flat, shape=(n, 3), strides=(stride_bytes, 8)).copy()


class GB300DPDServer:
    """Continuous-batching job server over the C ABI's ``pdpd_server_*`` (no counterpart in the
    reference, which runs one world per engine).

    ``submit(world, n_steps, on_interval=None)`` queues a job and returns its id; the world is
    copied.  ``on_interval(job_id, t, x, v, f)`` (optional) is called on the server's worker
    thread after every ``interval_steps`` steps of the job; returning ``False`` ends the job at
    that snapshot.  ``drain()`` waits for every queued job and raises the first error.  The
    final state of job ``i`` is ``results[i] = (x, v, f, t)``; failed jobs are in ``failed``.
    With ``keep_results=False`` the final states are not copied (``results[i] = t`` only) and
    snapshots are copied only for jobs with an ``on_interval`` handler.
    """

    def __init__(self, precision="fp32", device=-1, memory_budget_bytes=40 << 30,
                 interval_steps=100, keep_results=True):
        code = {"fp32": PDPD_FP32, "fp64": PDPD_FP64}[precision]
        h = C.c_void_p()
        rc = lib().pdpd_server_create(code, device, int(memory_budget_bytes), int(interval_steps),
                                      C.byref(h))
        if rc != 0:
            raise RuntimeError(f"pdpd_server_create: {STATUS.get(rc)}: "
                               f"{lib().pdpd_last_error(None).decode()}")
        self._h = h
        self.precision = precision
        self.interval_steps = int(interval_steps)
        self.keep_results = bool(keep_results)
        self.results = {}
        self.snapshots = {}   # job id -> number of interval callbacks seen
        self.failed = {}      # job id -> status name
        self._handlers = {}
        self._errors = []
        self._cb = JOB_FN(self._dispatch)

    def _dispatch(self, user, job, t, x, v, f, stride, n, status):
        try:
            if status < 0:
                self.failed[job] = STATUS.get(-status, -status)
                self._handlers.pop(job, None)
                return 0
            h = self._handlers.get(job)
            if not self.keep_results and h is None:
                if status == 1:
                    self.results[job] = int(t)
                else:
                    self.snapshots[job] = self.snapshots.get(job, 0) + 1
                return 1
            xs, vs, fs = _rows(x, n, stride), _rows(v, n, stride), _rows(f, n, stride)
            if status == 1:
                self.results[job] = (xs, vs, fs, int(t))
                self._handlers.pop(job, None)
                return 1
            self.snapshots[job] = self.snapshots.get(job, 0) + 1
            if h is not None and h(job, int(t), xs, vs, fs) is False:
                self.results[job] = (xs, vs, fs, int(t))
                self._handlers.pop(job, None)
                return 0
            return 1
        except BaseException as e:  # noqa: BLE001 -- re-raised by drain()
            self._errors.append(e)
            return 0

    def submit(self, world, n_steps, on_interval=None) -> int:
        fl = _Flat(world)
        jid = C.c_uint64(0)
        rc = lib().pdpd_server_submit(self._h, C.byref(fl.struct), int(n_steps), self._cb, None,
                                      C.byref(jid))
        if rc != 0:
            raise RuntimeError(f"submit: {STATUS.get(rc)}: {lib().pdpd_last_error(None).decode()}")
        if on_interval is not None:
            self._handlers[int(jid.value)] = on_interval
        return int(jid.value)

    def drain(self):
        rc = lib().pdpd_server_drain(self._h)
        if self._errors:
            e, self._errors = self._errors[0], []
            raise e
        if rc != 0:
            raise RuntimeError(f"drain: {STATUS.get(rc)}: {lib().pdpd_last_error(None).decode()}")

    def config(self, key, value):
        rc = lib().pdpd_server_config(self._h, str(key).encode(), str(value).encode())
        if rc != 0:
            raise RuntimeError(f"config: {STATUS.get(rc)}: {lib().pdpd_last_error(None).decode()}")

    def stats(self) -> dict:
        st = PdpdServerStats()
        lib().pdpd_server_stats_get(self._h, C.byref(st))
        return {n: getattr(st, n) for n, _ in PdpdServerStats._fields_ if n != "pad"}

    def kernel_launches(self):
        return int(lib().pdpd_kernel_launches(lib().pdpd_server_engine(self._h)))

    def close(self):
        if getattr(self, "_h", None):
            lib().pdpd_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
