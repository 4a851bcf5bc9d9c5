"""Build recipe for the oracle (test infrastructure only).

* ``build_oracle()`` compiles the C restatement ``oracle/mcrg_oracle.c`` into
  ``oracle/_build/liboracle.so`` (gcc, portable flags: it must build the same
  on x86-64 and aarch64).
* ``build_ref()`` compiles the reference's own unmodified sources
  (src/definitions.cpp, lattice.cpp, ising.cpp, mcrg.cpp, rgnn.cpp of kim-jane/MCRG,
  read where they lie under the reference checkout: ``$MCRG_REFERENCE_DIR``,
  by default ``/root/reference``) together with
  ``oracle/ref_harness.cpp`` and the single-rank ``oracle/stub_mpi/mpi.h``
  into ``oracle/_ref/libmcrg_ref.so``.  Nothing is copied out of the
  reference tree.  Only possible where the reference is mounted.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REF_ROOT = os.environ.get("MCRG_REFERENCE_DIR", "/root/reference")
REF_SRC = os.path.join(REF_ROOT, "src")
ORACLE_SO = os.path.join(HERE, "_build", "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libmcrg_ref.so")


def _newer(target: str, sources: list[str]) -> bool:
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(s) <= t for s in sources if os.path.exists(s))


def build_oracle(force: bool = False) -> str:
    src = os.path.join(HERE, "mcrg_oracle.c")
    if not force and _newer(ORACLE_SO, [src]):
        return ORACLE_SO
    os.makedirs(os.path.dirname(ORACLE_SO), exist_ok=True)
    tmp = ORACLE_SO + ".tmp%d" % os.getpid()
    cmd = ["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-fno-strict-aliasing", src, "-o", tmp, "-lm"]
    subprocess.check_call(cmd)
    os.replace(tmp, ORACLE_SO)
    return ORACLE_SO


def ref_available() -> bool:
    return os.path.isdir(REF_SRC)


def build_ref(force: bool = False) -> str | None:
    if not ref_available():
        return None
    units = [os.path.join(REF_SRC, f) for f in ("definitions.cpp", "lattice.cpp", "ising.cpp", "mcrg.cpp", "rgnn.cpp")]
    harness = os.path.join(HERE, "ref_harness.cpp")
    if not force and _newer(REF_SO, units + [harness]):
        return REF_SO
    os.makedirs(os.path.dirname(REF_SO), exist_ok=True)
    tmp = REF_SO + ".tmp%d" % os.getpid()
    cmd = ["g++", "-std=c++14", "-O3", "-fPIC", "-shared", "-w",
           "-I", os.path.join(HERE, "stub_mpi"), "-I", REF_SRC] + units + [harness, "-o", tmp]
    subprocess.check_call(cmd)
    os.replace(tmp, REF_SO)
    return REF_SO


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
    print(build_ref(force="--force" in sys.argv))
