"""The reference's own call sites compile unchanged against the GPU drop-in.

kim-jane/MCRG's src/main.cpp (MonteCarloRenormalizationGroup::
calc_critical_exponent), src/train.cpp and src/rgnn.cpp (which hands
Lattice::spins_ to Eigen code as an `imat`, src/rgnn.cpp:113-114,175) are
compiled as they are in the reference checkout, with mcrg_gb300/shim/dropin's
headers in place of the reference's, and linked with libmcrg.so.  Runs where
the reference is mounted (MCRG_REFERENCE_DIR, default /root/reference); the
single-rank MPI header of oracle/stub_mpi stands in for an MPI installation.
"""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.environ.get("MCRG_REFERENCE_DIR", "/root/reference")


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "src")), reason="reference checkout not mounted")
def test_reference_main_train_rgnn_build_against_dropin(mcrg_lib):
    import sys
    sys.path.insert(0, os.path.join(ROOT, "mcrg_gb300", "shim", "dropin"))
    import build as dropin_build
    bins = dropin_build.build(REF, os.path.join(ROOT, "oracle", "stub_mpi"))
    for name in ("run", "train"):
        assert os.path.isfile(bins[name]) and os.access(bins[name], os.X_OK)
        syms = subprocess.run(["nm", "-D", "--undefined-only", bins[name]], capture_output=True, text=True).stdout
        assert "mcrg_alloc" in syms  # the reference's calls land in libmcrg
    # the reference's own Lattice / IsingModel / MCRG implementations are not in the binaries
    for name in ("run", "train"):
        out = subprocess.run(["nm", "-C", bins[name]], capture_output=True, text=True).stdout
        assert "Lattice::Lattice(int)" not in out
        assert "IsingModel::grow_cluster" not in out
