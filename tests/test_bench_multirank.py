"""bench.py's multi-rank path on CPU (gloo, world size 2).

`bench.py --gpus N` runs one rank per GPU (replica = rank) and adds the
ranks' exact moment sums with bench.replica_sum, as MPI_Allreduce(SUM) does
in the reference (src/mcrg.cpp:101-103).  Here each rank's chain comes from
the oracle (no GPU): the sum over two gloo ranks, formed by the bench's own
Dist and replica_sum, must equal one process adding both chains.
"""
import os
import socket

import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, out_q):
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "RANK": str(rank),
                       "LOCAL_RANK": str(rank), "WORLD_SIZE": str(world)})
    import bench
    from oracle import oracle as O
    from mcrg_gb300.tmatrix import MomentSums
    D = bench.Dist()
    assert (D.rank, D.world) == (rank, world)
    tr, _ = O.chain(32, bench.KC, 5, 4, 1, rank, n_eq=10, n_samples=12, sweeps_between=2)
    total = bench.replica_sum(MomentSums.from_trace(tr))
    D.barrier()
    if rank == 0:
        out_q.put((total.n_samples, total.S, total.SbS, total.SbSb))
    D.pg.destroy_process_group()


def test_bench_replica_sum_over_two_gloo_ranks():
    import bench
    from oracle import oracle as O
    from mcrg_gb300.tmatrix import MomentSums
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = q.get(timeout=300)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    ref = None
    for r in range(2):
        tr, _ = O.chain(32, bench.KC, 5, 4, 1, r, n_eq=10, n_samples=12, sweeps_between=2)
        m = MomentSums.from_trace(tr)
        ref = m if ref is None else ref + m
    assert got == (ref.n_samples, ref.S, ref.SbS, ref.SbSb)


def test_single_process_sum_is_identity():
    import bench
    from oracle import oracle as O
    from mcrg_gb300.tmatrix import MomentSums
    tr, _ = O.chain(16, bench.KC, 2, 3, 4, 0, n_eq=5, n_samples=6)
    m = MomentSums.from_trace(tr)
    assert bench.replica_sum(m) == m


def test_cpu_threads_fit_memory():
    import bench
    n, why = bench.cpu_threads(16384)
    assert 1 <= n <= (os.cpu_count() or 1) and why
