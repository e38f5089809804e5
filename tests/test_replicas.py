"""The multi-GPU form of the bench is replicas only (images are independent,
the path has no exchange step): each rank denoises its own batch and the job
time is the slowest rank's.  This checks that timing logic on CPU with two
gloo ranks (no GPU involved)."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(('127.0.0.1', 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, results):
    os.environ.update(MASTER_ADDR='127.0.0.1', MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import torch.distributed as dist
    import bench
    dist.init_process_group('gloo', rank=rank, world_size=world)
    try:
        ms = 100.0 + 25.0 * rank  # rank 1 is the slower replica
        results[rank] = (bench.max_over_ranks(ms, 'cpu'), bench.dist_env()[:2])
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_two_gloo_ranks():
    ctx = mp.get_context('spawn')
    with ctx.Manager() as m:
        results = m.dict()
        port = _free_port()
        procs = [ctx.Process(target=_rank_main, args=(r, 2, port, results)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        res = dict(results)
    assert res[0][0] == res[1][0] == 125.0
    assert res[0][1] == (0, 2) and res[1][1] == (1, 2)


def test_single_process_and_throughput():
    import bench
    assert bench.max_over_ranks(42.0, 'cpu') == 42.0
    # 2 replicas of 64 images each in 0.5 s of job time
    assert bench.job_throughput(64, 2, 0.5) == pytest.approx(256.0)
