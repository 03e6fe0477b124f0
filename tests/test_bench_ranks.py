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


def test_reference_arm_line_keeps_the_contract():
    """bench.py --impl reference on the host: one JSON line with the arm's
    metric and config, a cpu_baseline describing the run and an e2e equal
    to it with no host-device bytes; rank 1 of a 2-rank launch prints
    nothing.  (The small linear-map workload keeps the test short.)"""
    import json
    import subprocess
    cmd = [sys.executable, os.path.join(ROOT, 'bench.py'), '--impl',
           'reference', '--steps', '3', '--warmup', '3', '--workload', 'c1']
    out = subprocess.run(cmd, capture_output=True, text=True, timeout=600,
                         cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.startswith('{')]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d['impl'] == 'reference'
    assert d['unit'] == 'macroparticle-turns/s' and d['higher_is_better']
    assert d['value'] > 0 and d['steps'] == 3 and d['warmup'] == 3
    # the same workload description as the GPU arm's line
    sys.path.insert(0, ROOT)
    import bench
    assert d['config'] == bench.bench_config(bench.WORKLOADS['c1'])
    cb = d['cpu_baseline']
    assert cb['value'] == d['value'] and cb['cores'] >= 1
    assert cb['kind'] in ('port', 'reference') and cb['sample']
    assert cb['host']['logical_cpus'] >= 1 and cb['host']['machine']
    assert d['e2e'] == {'value': d['value'], 'unit': d['unit'],
                        'h2d_bytes_per_step': 0, 'd2h_bytes_per_step': 0}
    env = dict(os.environ, WORLD_SIZE='2', RANK='1', LOCAL_RANK='1')
    out = subprocess.run(cmd, capture_output=True, text=True, timeout=600,
                         cwd=ROOT, env=env)
    assert out.returncode == 0, out.stderr[-2000:]
    assert not [l for l in out.stdout.splitlines() if l.startswith('{')]


def test_host_description_never_raises(monkeypatch):
    """The CPU baseline's host record: architecture, logical CPUs and the
    model from /proc/cpuinfo, or None when that cannot be read."""
    import builtins
    sys.path.insert(0, ROOT)
    import bench
    h = bench.host_cpu()
    assert set(h) == {'machine', 'logical_cpus', 'model', 'OMP_NUM_THREADS',
                      'OPENBLAS_NUM_THREADS'}
    real_open = builtins.open

    def no_cpuinfo(path, *a, **k):
        if path == '/proc/cpuinfo':
            raise OSError('unreadable')
        return real_open(path, *a, **k)
    monkeypatch.setattr(builtins, 'open', no_cpuinfo)
    assert bench.host_cpu()['logical_cpus'] == h['logical_cpus']
