"""The DPDEngine adapter (poets-dpd_gb300/host) compiled against the reference's own headers:
it registers with the reference's DPDEngineFactory, answers CanSupport through the reference's
base checks, and flattens a WorldState exactly as the Python mirror (pdpd_world.World) does.
Needs the reference sources (skipped where they are absent); touches no GPU."""

import os
import struct
import subprocess

import numpy as np
import pytest

import pdpd_world as W
import v2binary as V
from _helpers import load_v2_fixture, v2_fixture_names

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _reference_include():
    """PDPD_REFERENCE_INCLUDE, else what the reference build recipe (oracle/ref/Makefile)
    reports: the reference's include directory, or nothing where the sources are absent."""
    if os.environ.get("PDPD_REFERENCE_INCLUDE"):
        return os.environ["PDPD_REFERENCE_INCLUDE"]
    try:
        r = subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle", "ref"),
                            "print-include"], capture_output=True, text=True, timeout=60)
        return r.stdout.strip()
    except (OSError, subprocess.TimeoutExpired):
        return ""


REF_INCLUDE = _reference_include()
BUILD = os.path.join(ROOT, "poets-dpd_gb300", "_build")
EXE = os.path.join(BUILD, "adapter_check")

pytestmark = pytest.mark.skipif(not REF_INCLUDE or not os.path.isdir(os.path.join(REF_INCLUDE, "dpd")),
                                reason="reference sources not present")


@pytest.fixture(scope="module")
def exe():
    lib_dir = os.path.join(ROOT, "poets-dpd_gb300")
    if not os.path.exists(os.path.join(lib_dir, "libpdpd_gb300.so")):
        import build as B
        B.build()
    os.makedirs(BUILD, exist_ok=True)
    cmd = ["g++", "-std=c++17", "-O1", "-w", "-I" + REF_INCLUDE, "-I" + os.path.join(ROOT, "include"),
           "-I" + os.path.join(ROOT, "poets-dpd_gb300", "host"), "-I" + os.path.join(ROOT, "oracle", "ref"),
           os.path.join(ROOT, "tests", "adapter_check.cpp"),
           os.path.join(ROOT, "poets-dpd_gb300", "host", "gb300_dpd_engine.cpp"),
           "-L" + lib_dir, "-lpdpd_gb300", "-Wl,-rpath," + lib_dir, "-o", EXE]
    subprocess.run(cmd, check=True)
    return EXE


def run(exe, *args):
    r = subprocess.run([exe, *args], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return r.stdout


def test_registers_with_the_reference_factory(exe):
    names = run(exe, "factories").split()
    assert "gb300_dpd_engine_fp32" in names and "gb300_dpd_engine_fp64" in names


def test_can_support(exe, tmp_path):
    p = tmp_path / "w.pdw1"
    W.write_pdw1(W.make_polymer_box(8, chain_fraction=0.1), str(p))
    out = run(exe, "cansupport", "gb300_dpd_engine_fp32", str(p))
    assert "[]" in out and "max_bond_length 2" in out
    w = W.make_water(4)
    w.stationary = np.array([True])  # stationary bead types are supported
    W.write_pdw1(w, str(p))
    out = run(exe, "cansupport", "gb300_dpd_engine_fp64", str(p))
    assert "[]" in out
    w = W.make_water(4)
    w.box = np.array([4, 1, 4], np.int32)
    W.write_pdw1(w, str(p))
    out = run(exe, "cansupport", "gb300_dpd_engine_fp64", str(p))
    assert "at least 2" in out


def read_vectors(path):
    data = open(path, "rb").read()
    p, out = 0, []
    kinds = ["<u4", "<f8", "<f8", "<u4", "<f8", "<f8", "<u4", "<f8", "<f8", "<f8", "<f8"]
    for k in kinds:
        (n,) = struct.unpack_from("<Q", data, p)
        p += 8
        size = np.dtype(k).itemsize
        out.append(np.frombuffer(data, k, n, p))
        p += n * size
    return out


def test_flatten_matches_python_mirror(exe, tmp_path):
    world = W.make_polymer_box(10, chain_fraction=0.1, seed=4)
    world.t = 17
    p = tmp_path / "w.pdw1"
    W.write_pdw1(world, str(p))
    out = tmp_path / "flat.bin"
    run(exe, "flatten", str(p), str(out))
    hash_, cons, diss, bb, bk, br, ab, ak, at, head, x = read_vectors(str(out))
    pbb, pbk, pbr, pab, pak, pat = world.flat_bonds()
    assert np.array_equal(hash_, world.hashes())
    assert np.array_equal(cons, world.conservative.reshape(-1))
    assert np.array_equal(diss, world.dissipative.reshape(-1))
    assert np.array_equal(bb, pbb.reshape(-1)) and np.array_equal(bk, pbk) and np.array_equal(br, pbr)
    assert np.array_equal(ab, pab.reshape(-1)) and np.array_equal(ak, pak) and np.array_equal(at, pat)
    assert list(head[:3]) == list(world.box) and head[5] == 17 and head[6] == world.n_beads
    assert head[7] == 88  # sizeof(Bead): x/v/f read in place from the reference's beads
    assert np.array_equal(x.reshape(-1, 3), world.x)


@pytest.mark.parametrize("name", v2_fixture_names())
def test_v2binary_file_writer_matches_reference(exe, tmp_path, name):
    """gb300_v2binary.hpp writes the reference's text header around a GPU-encoded section:
    with the reference's own section, the file equals the reference writer's byte for byte."""
    world, v2, _, _, _ = load_v2_fixture(name)
    _, section = V.split_file(v2)
    pw, ps, po = tmp_path / "w.pdw1", tmp_path / "s.bin", tmp_path / "o.v2"
    W.write_pdw1(world, str(pw))
    ps.write_bytes(section)
    run(exe, "v2file", str(pw), str(ps), str(po))
    assert po.read_bytes() == v2


@pytest.mark.parametrize("name", ["merge_spatial_water", "merge_spatial_polymer"])
def test_spatial_parameters_flatten_to_the_reference_cell_values(exe, tmp_path, name):
    """Spatially varying strengths pass CanSupport and flatten into per-cell tables equal to
    the values the reference itself evaluates per cell (ref_harness tables)."""
    d = np.load(os.path.join(ROOT, "tests", "golden", name + ".npz"))
    world = W.read_pdw1(d["world"].tobytes())
    pw, pe, po = tmp_path / "w.pdw1", tmp_path / "e.txt", tmp_path / "o.bin"
    W.write_pdw1(world, str(pw))
    pe.write_text("\n".join(str(x) for x in d["exprs"]) + "\n")
    out = run(exe, "spatial", str(pw), str(pe), str(po))
    assert "[]" in out
    data = po.read_bytes()
    (n,) = struct.unpack_from("<Q", data, 0)
    ca = np.frombuffer(data, "<f8", n, 8)
    (m,) = struct.unpack_from("<Q", data, 8 + 8 * n)
    cg = np.frombuffer(data, "<f8", m, 16 + 8 * n)
    assert np.array_equal(ca, d["cell_a"].reshape(-1)) and np.array_equal(cg, d["cell_g"].reshape(-1))
