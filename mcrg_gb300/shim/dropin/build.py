"""Builds the reference's own call sites against the GPU drop-in.

kim-jane/MCRG's src/main.cpp, src/train.cpp and src/rgnn.cpp are compiled
unmodified, where they lie in the reference checkout, with the headers of
this directory (lattice.hpp, ising.hpp, mcrg.hpp) taking the place of the
reference's: a build directory holds symbolic links to the reference's
sources and headers, plus links to these drop-in headers under the
reference's header names, so every quote include of the reference resolves
to the drop-in.  The reference's definitions.cpp (random generators, helpers)
and vendored Eigen are used as they are.  The objects link with the GPU
classes (mcrg_gb300/shim/mcrg_classes.cpp built with MCRG_EIGEN_SPINS: spins_
is the reference's Eigen `imat`) and libmcrg.so into `run` (src/main.cpp)
and `train` (src/train.cpp + src/rgnn.cpp).

    python mcrg_gb300/shim/dropin/build.py [reference checkout] [mpi include dir]

The MPI header is the system's (`mpicxx` users) or, for a single-process
build, any <mpi.h> on the include path given as the second argument.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SHIM = os.path.dirname(HERE)
PKG = os.path.dirname(SHIM)
OUT = os.path.join(PKG, "_build", "dropin")
REFERENCE_SOURCES = ("main.cpp", "train.cpp", "rgnn.cpp", "rgnn.hpp", "definitions.cpp", "definitions.hpp", "Eigen")
DROPIN_HEADERS = ("lattice.hpp", "ising.hpp", "mcrg.hpp")


def _link(src: str, dst: str) -> None:
    if os.path.lexists(dst):
        os.remove(dst)
    os.symlink(src, dst)


def build(reference: str, mpi_include: str | None = None, out: str = OUT) -> dict:
    """Compiles and links; returns {"run": path, "train": path}."""
    from mcrg_gb300 import build as B
    lib = B.build()
    ref_src = os.path.join(reference, "src")
    src = os.path.join(out, "src")
    os.makedirs(src, exist_ok=True)
    for f in REFERENCE_SOURCES:
        _link(os.path.join(ref_src, f), os.path.join(src, f))
    for f in DROPIN_HEADERS:
        _link(os.path.join(HERE, f), os.path.join(src, f))
    flags = ["-std=c++17", "-O2", "-w", "-DMCRG_EIGEN_SPINS=1", "-I", SHIM, "-I", src]
    if mpi_include:
        flags += ["-I", mpi_include]
    objs = {}
    units = [(os.path.join(src, f + ".cpp"), f) for f in ("main", "train", "rgnn", "definitions")]
    units.append((os.path.join(SHIM, "mcrg_classes.cpp"), "mcrg_classes"))
    for path, name in units:
        obj = os.path.join(out, name + ".o")
        r = subprocess.run(["g++"] + flags + ["-c", path, "-o", obj], capture_output=True, text=True)
        if r.returncode:
            raise RuntimeError("compiling %s failed:\n%s" % (path, r.stderr))
        objs[name] = obj
    libdir = os.path.dirname(lib)
    link = ["-L", libdir, "-lmcrg", "-Wl,-rpath," + libdir]
    bins = {}
    for name, parts in (("run", ("main", "definitions", "mcrg_classes")),
                        ("train", ("train", "rgnn", "definitions", "mcrg_classes"))):
        exe = os.path.join(out, name)
        r = subprocess.run(["g++"] + [objs[p] for p in parts] + link + ["-o", exe], capture_output=True, text=True)
        if r.returncode:
            raise RuntimeError("linking %s failed:\n%s" % (name, r.stderr))
        bins[name] = exe
    return bins


if __name__ == "__main__":
    sys.path.insert(0, os.path.dirname(PKG))
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("MCRG_REFERENCE_DIR", "/root/reference")
    print(build(ref, sys.argv[2] if len(sys.argv) > 2 else None))
