"""Sharded bunch and bunch packing, host side (no GPU).

* shard_range covers the bunch with contiguous, balanced, disjoint ranges;
* pack_bunches: every bunch on exactly one rank, greedy largest-first
  packing, and the load spread of the greedy bound;
* two gloo ranks (world_size 2, one process each): each folds its block of
  a bunch's partial slice columns into compensated sums (the host
  restatement of phk_slice_sums), the ranks all-gather them through
  Shards, and the rank-ordered merge gives, on both ranks, bit for bit
  the totals of one rank folding every column -- and the correctly
  rounded sums of the columns (math.fsum).
"""
import math
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip('torch')
dist = pytest.importorskip('torch.distributed')


def test_shard_range():
    from pyheadtail_gb300.shards import shard_range
    for n in (0, 1, 7, 10**7 + 3):
        for world in (1, 2, 3, 8):
            r = [shard_range(n, k, world) for k in range(world)]
            assert r[0][0] == 0 and r[-1][1] == n
            for (a, b), (c, d) in zip(r, r[1:]):
                assert b == c
            sizes = [b - a for a, b in r]
            assert max(sizes) - min(sizes) <= 1
            assert sizes == sorted(sizes, reverse=True)
    with pytest.raises(ValueError):
        shard_range(10, 2, 2)


def test_pack_bunches():
    from pyheadtail_gb300.shards import pack_bunches
    rng = np.random.RandomState(3)
    sizes = rng.randint(10**5, 4 * 10**5, size=256)
    for world in (1, 2, 3, 8):
        packs = pack_bunches(sizes, world)
        flat = sorted(b for p in packs for b in p)
        assert flat == list(range(len(sizes)))
        loads = [int(sizes[p].sum()) if p else 0 for p in packs]
        # greedy largest-first: the spread is at most the largest bunch
        assert max(loads) - min(loads) <= int(sizes.max())
        assert all(p == sorted(p) for p in packs)
    assert pack_bunches([5, 3, 3, 1], 2) == [[0, 3], [1, 2]]


def _columns(S=200, G=300, seed=11):
    rng = np.random.RandomState(seed)
    counts = rng.randint(0, 50, size=(S, G)).astype(np.float64)
    sx = rng.normal(0, 1e-3, size=(S, G)) * counts
    sy = rng.normal(0, 1e-3, size=(S, G)) * counts
    sx[5] *= 1e9        # wide dynamic range in one slice
    sx[6, ::7] = -sx[6, 1::7][:sx[6, ::7].size]     # cancellation
    return np.stack([counts, sx, sy])


def _worker(rank, world, port, out_dir):
    os.environ['MASTER_ADDR'] = '127.0.0.1'
    os.environ['MASTER_PORT'] = str(port)
    import sys
    here = os.path.dirname(os.path.abspath(__file__))
    sys.path.insert(0, os.path.dirname(here))
    sys.path.insert(0, here)
    import torch.distributed as d
    import shard_host as H
    from pyheadtail_gb300.shards import Shards, shard_range
    d.init_process_group('gloo', rank=rank, world_size=world)
    try:
        P = _columns()
        G = P.shape[2]
        g0, g1 = shard_range(G, rank, world)
        local = torch.from_numpy(H.fold_columns(P[:, :, g0:g1]))
        sh = Shards()
        assert (sh.rank, sh.world) == (rank, world)
        gathered = sh.all_gather(local).numpy()
        totals = H.merge_pairs(gathered)
        np.save(os.path.join(out_dir, 'tot%d.npy' % rank), totals)
        np.save(os.path.join(out_dir, 'gat%d.npy' % rank), gathered)
    finally:
        d.destroy_process_group()


def _free_port():
    s = socket.socket()
    s.bind(('127.0.0.1', 0))
    p = s.getsockname()[1]
    s.close()
    return p


def test_rank_ordered_merge_equals_single_rank(tmp_path):
    import torch.multiprocessing as mp
    import shard_host as H
    world = 2
    mp.start_processes(_worker, args=(world, _free_port(), str(tmp_path)),
                       nprocs=world, start_method='spawn', join=True)
    P = _columns()
    single = H.merge_pairs(H.fold_columns(P)[None])
    t0 = np.load(str(tmp_path / 'tot0.npy'))
    t1 = np.load(str(tmp_path / 'tot1.npy'))
    g0 = np.load(str(tmp_path / 'gat0.npy'))
    g1 = np.load(str(tmp_path / 'gat1.npy'))
    assert g0.tobytes() == g1.tobytes()
    assert t0.tobytes() == t1.tobytes()
    assert t0.tobytes() == single.tobytes()
    exact = np.array([[math.fsum(P[q, s]) for s in range(P.shape[1])]
                      for q in range(3)])
    assert t0.tobytes() == exact.tobytes()
    # the plain fixed-order FP64 fold is within rounding of it
    plain = P.sum(axis=2)
    np.testing.assert_allclose(plain[1], exact[1], rtol=1e-12,
                               atol=1e-15 * np.abs(P[1]).sum(axis=1).max())
    n, mx, my, mom = H.finalize(t0)
    np.testing.assert_array_equal(n, P[0].sum(axis=1).astype(np.int32))


def test_single_shard_without_process_group():
    from pyheadtail_gb300.shards import Shards
    if dist.is_initialized():
        pytest.skip('a process group is initialised in this process')
    sh = Shards()
    assert (sh.rank, sh.world) == (0, 1)
    t = torch.arange(6.0).reshape(2, 3)
    assert torch.equal(sh.all_gather(t)[0], t)
    assert sh.range(11) == (0, 11)
