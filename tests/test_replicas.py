"""Multi-GPU is replicas only: every rank meshes its own volume, no data-path
collective.  The only exchange is the benchmark's max-over-ranks of the step times;
here two gloo ranks on the CPU run it, as torchrun would launch them."""
import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(('127.0.0.1', 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    os.environ.update(MASTER_ADDR='127.0.0.1', MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import torch.distributed as dist
    import bench
    dist.init_process_group('gloo', rank=rank, world_size=world)
    try:
        # rank r: device step 2 + r ms, end to end 40 - r ms
        ms, e2e = bench.max_over_ranks(dist, [2.0 + rank, 40.0 - rank], 'cpu')
        dist.barrier()
        q.put((rank, ms, e2e, bench.whole_job_rate(1024 ** 3, world, ms)))
    finally:
        dist.destroy_process_group()


def test_two_replicas_report_the_slowest_rank():
    import torch.multiprocessing as mp
    ctx = mp.get_context('spawn')
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, ms, e2e, rate in got:
        assert (ms, e2e) == (3.0, 40.0)  # max over the ranks, on every rank
        assert rate == pytest.approx(2 * 1024 ** 3 / 3e-3)  # both replicas' voxels in the slowest time


def test_single_process_is_the_identity():
    import bench
    assert bench.max_over_ranks(None, [1.5, 2.5]) == [1.5, 2.5]
    assert bench.whole_job_rate(10, 1, 2.0) == pytest.approx(5000.0)
