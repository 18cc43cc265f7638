"""Build recipe of the engine's shared library (libpdpd_gb300.so), for sm_103a only.

Compiles the kernel translation units with nvcc (-gencode arch=compute_103a,code=sm_103a,
-lineinfo), the host runtime with g++, in parallel, and links them in-tree.  The FP64
kernels are compiled with -fmad=false so that no multiply-add is fused (bit-exact FP64).
"""

from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libpdpd_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _cuda_home(nvcc):
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def build(verbose: bool = False) -> str:
    nvcc = _nvcc()
    cuda = _cuda_home(nvcc)
    os.makedirs(BUILD, exist_ok=True)
    common = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xptxas", "-v"] + ARCH
    jobs = [
        [nvcc] + common + ["-c", os.path.join(CSRC, "pdpd_fp32.cu"), "-o", os.path.join(BUILD, "pdpd_fp32.o")],
        [nvcc] + common + ["-fmad=false", "-c", os.path.join(CSRC, "pdpd_fp64.cu"), "-o", os.path.join(BUILD, "pdpd_fp64.o")],
        [nvcc] + common + ["-c", os.path.join(CSRC, "pdpd_sort.cu"), "-o", os.path.join(BUILD, "pdpd_sort.o")],
        [nvcc] + common + ["-fmad=false", "-c", os.path.join(CSRC, "pdpd_observe.cu"), "-o",
                           os.path.join(BUILD, "pdpd_observe.o")],
        [nvcc] + common + ["-fmad=false", "-c", os.path.join(CSRC, "pdpd_codec.cu"), "-o",
                           os.path.join(BUILD, "pdpd_codec.o")],
        [nvcc] + common + ["-c", os.path.join(CSRC, "pdpd_hostio.cu"), "-o", os.path.join(BUILD, "pdpd_hostio.o")],
        [nvcc] + common + ["-c", os.path.join(CSRC, "pdpd_bondcsr.cu"), "-o", os.path.join(BUILD, "pdpd_bondcsr.o")],
        ["g++", "-O2", "-std=c++17", "-fPIC", "-Wall", "-I" + os.path.join(cuda, "include"),
         "-c", os.path.join(CSRC, "pdpd_engine.cpp"), "-o", os.path.join(BUILD, "pdpd_engine.o")],
    ]
    with cf.ThreadPoolExecutor(len(jobs)) as ex:
        logs = list(ex.map(_run, jobs))
    objs = [os.path.join(BUILD, n) for n in ("pdpd_fp32.o", "pdpd_fp64.o", "pdpd_sort.o",
                                              "pdpd_observe.o", "pdpd_codec.o", "pdpd_hostio.o",
                                              "pdpd_bondcsr.o", "pdpd_engine.o")]
    tmp = LIB + ".tmp"
    _run([nvcc, "-shared"] + ARCH + objs + ["-o", tmp, "-lcudart"])
    os.replace(tmp, LIB)
    log = "\n".join(logs)
    if verbose:
        print(log)
    return log


if __name__ == "__main__":
    build(verbose=True)
