"""Builds libmcrg.so (the CUDA hot path + C ABI) for sm_103a, in-tree.

Each translation unit is compiled by its own nvcc process (in parallel) and
the objects are linked into ``mcrg_gb300/_build/libmcrg.so``.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libmcrg.so")
UNITS = ["mcrg_chain.cu", "mcrg_tiled.cu", "mcrg_capi.cu", "mcrg_batch.cu", "mcrg_noalloc.cu", "mcrg_rgnn.cu",
         "mcrg_cluster.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
                     "--expt-relaxed-constexpr"]


def _nvcc() -> str:
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else "nvcc"


def _sources() -> list[str]:
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cu", ".cuh"))] + [
        os.path.join(HERE, "..", "include", "mcrg.h")]


def up_to_date() -> bool:
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(s) <= t for s in _sources())


def build(force: bool = False, verbose: bool = False, extra: list[str] | None = None) -> str:
    if not force and up_to_date():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    nvcc = _nvcc()
    flags = NVCC_FLAGS + (extra or [])

    def compile_unit(u: str) -> str:
        obj = os.path.join(OUT_DIR, u.replace(".cu", ".o"))
        cmd = [nvcc] + flags + ["-c", os.path.join(CSRC, u), "-o", obj]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s%s" % (u, r.stdout, r.stderr))
        if verbose and (r.stdout or r.stderr):
            print(r.stdout + r.stderr, flush=True)
        return obj

    with cf.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        objs = list(ex.map(compile_unit, UNITS))
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = [nvcc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart", "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s%s" % (r.stdout, r.stderr))
    os.replace(tmp, LIB)
    return LIB


SHIM = os.path.join(HERE, "shim")
SHIM_BIN = os.path.join(OUT_DIR, "run_mcrg")


def build_shim(force: bool = False) -> str:
    """The reference-named C++ classes + the src/main.cpp-style driver,
    linked against libmcrg.so (g++, host code only)."""
    lib = build()
    srcs = [os.path.join(SHIM, f) for f in ("mcrg_classes.cpp", "run_mcrg.cpp")]
    deps = srcs + [os.path.join(SHIM, f) for f in ("mcrg_classes.hpp", "tmatrix.hpp")] + [lib]
    if not force and os.path.exists(SHIM_BIN) and all(os.path.getmtime(d) <= os.path.getmtime(SHIM_BIN)
                                                      for d in deps):
        return SHIM_BIN
    tmp = SHIM_BIN + ".tmp%d" % os.getpid()
    # no FMA contraction: the log files reproduce the reference's double arithmetic
    cmd = ["g++", "-O2", "-std=c++17", "-ffp-contract=off"] + srcs + ["-L", OUT_DIR, "-lmcrg", "-Wl,-rpath,$ORIGIN", "-o", tmp]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("shim build failed:\n%s%s" % (r.stdout, r.stderr))
    os.replace(tmp, SHIM_BIN)
    return SHIM_BIN


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv,
                extra=["-Xptxas", "-v"] if "--ptxas" in sys.argv else None))
    print(build_shim(force="--force" in sys.argv))
