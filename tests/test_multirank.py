"""Multi-process replica path on CPU (gloo, world size 2).

Each rank runs the oracle chain for its own replicas and the exact moment
sums are combined across ranks, as MPI_Allreduce does in the reference
(src/mcrg.cpp:101-103).  The combined sums must equal one process summing
all replicas; sample splitting follows src/definitions.cpp:79-87.
"""
import os
import socket

import pytest
import torch.multiprocessing as mp

from mcrg_gb300.dist import replica_ids, split_samples


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, n_rep, out_q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from oracle import oracle as O
    from mcrg_gb300.dist import allreduce_moments
    from mcrg_gb300.tmatrix import MomentSums
    total = None
    for r in replica_ids(rank, world, n_rep):
        tr, _ = O.chain(16, -0.4406868, 3, 3, 77, r, n_eq=20, n_samples=15, sweeps_between=1)
        m = MomentSums.from_trace(tr)
        total = m if total is None else total + m
    total = allreduce_moments(total)
    dist.barrier()
    if rank == 0:
        out_q.put((total.n_samples, total.S, total.SbS, total.SbSb))
    dist.destroy_process_group()


def test_split_samples_matches_reference_rule():
    # rank 0 takes the remainder (src/definitions.cpp:79-87)
    assert [split_samples(r, 4, 10) for r in range(4)] == [1, 3, 3, 3]
    assert sum(split_samples(r, 3, 100) for r in range(3)) == 100
    assert split_samples(0, 8, 5) == -2  # the reference's quirk: can be <= 0


def test_replica_sum_over_two_gloo_ranks():
    from oracle import oracle as O
    from mcrg_gb300.tmatrix import MomentSums
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    n_rep = 5
    procs = [ctx.Process(target=_worker, args=(r, 2, port, n_rep, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = q.get(timeout=300)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    ref = None
    for r in range(n_rep):
        tr, _ = O.chain(16, -0.4406868, 3, 3, 77, r, n_eq=20, n_samples=15, sweeps_between=1)
        m = MomentSums.from_trace(tr)
        ref = m if ref is None else ref + m
    assert got == (ref.n_samples, ref.S, ref.SbS, ref.SbSb)
