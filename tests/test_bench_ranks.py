"""Host logic of bench.py's multi-GPU line, on CPU: with N replicas the
slowest rank's step time defines the whole-job throughput.  Two gloo ranks
on 127.0.0.1 stand in for the NCCL ranks of a GPU run."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR='127.0.0.1', MASTER_PORT=str(port))
    dist.init_process_group('gloo', rank=rank, world_size=world)
    try:
        ms = bench.max_over_ranks(1.5 + rank, world)
        out.put((rank, ms, bench.job_value(1000, ms, world)))
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_and_job_value_two_gloo_ranks():
    mp = pytest.importorskip('torch.multiprocessing')
    ctx = mp.get_context('spawn')
    q = ctx.Queue()
    port = 29500 + os.getpid() % 1000
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, ms, v in res:
        assert ms == 2.5                      # the slower rank's time
        assert v == pytest.approx(2 * 1000 / 2.5e-3)


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(3.25, 1) == 3.25
    assert bench.job_value(500, 2.0, 1) == pytest.approx(2.5e5)
