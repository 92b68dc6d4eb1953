"""The multi-GPU form of the benchmark without GPUs: ranks are independent replicas (their own seeded matrices, no
collective on the data path), the job time is the maximum over ranks, the whole-job rate counts every rank's
matrices.  Two gloo ranks on the CPU run the same reduction bench.py runs over nccl."""
import os

import numpy as np
import pytest
import torch.multiprocessing as mp


def _rank(rank, world, port, out):
    import torch.distributed as dist

    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms = 10.0 + 5.0 * rank  # rank 1 is the slower one
        worst = bench.max_over_ranks(ms, world, device="cpu")
        out[rank] = (worst, bench.whole_job_rate(1000, worst, world), bench.rank_seed(rank))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_reduce_like_the_benchmark():
    import socket
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        res = dict(out)
    assert res[0][0] == res[1][0] == 15.0                       # the slowest rank's time on every rank
    assert res[0][1] == pytest.approx(2 * 1000 / 15e-3)          # every rank's matrices over that time
    assert res[0][2] != res[1][2]                                # independent replicas


def test_replica_workloads_differ_and_repeat():
    from matfun_gb300 import workloads as w

    import bench
    a, b = (w.c1_gmf_groups(64, seed=bench.rank_seed(r)) for r in (0, 1))
    assert not np.array_equal(a, b)
    assert np.array_equal(a, w.c1_gmf_groups(64, seed=bench.rank_seed(0)))
