"""Sharded single bunch on the GPU (pyheadtail_gb300.shards).

* phk_slice_sums and phk_slice_merge equal their host restatement
  (tests/shard_host.py) bit for bit on random partial columns, and the
  merged totals are the correctly rounded sums of the columns;
* the multi-turn wake physics (RF, resonator + 50-turn resistive wall,
  500 slices, fixed cuts) on a bunch split into two shards: the shards
  run as two threads on this GPU, each with its own Particles, exchanging
  their slice sums through an in-process all-gather in rank order (there
  is one GPU per call here; between GPUs the same exchange is an NCCL
  all-gather).  Every turn both shards see the same slice counts and
  moments, the counts equal the unsharded bunch's, and after 20 turns
  the shards' coordinates equal the unsharded bunch's within 1e-12 of
  each coordinate's RMS (the slice sums differ from the unsharded fold
  by their rounding only)."""
import ctypes
import math
import threading

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip('torch')

N_TURNS = 20


def test_slice_sums_and_merge_match_host():
    import shard_host as H
    from pyheadtail_gb300 import _native as N
    from pyheadtail_gb300._engine import DeviceSlicer, stream_handle
    rng = np.random.RandomState(5)
    S, G = 300, 457
    counts = rng.randint(0, 40, size=(S, G)).astype(np.float64)
    P = np.stack([counts, rng.normal(0, 1e-3, (S, G)) * counts,
                  rng.normal(0, 1e6, (S, G)) * counts])
    parts = torch.from_numpy(P.reshape(-1).copy()).cuda()
    ds = DeviceSlicer(-0.5, 0.5, S, N.PHK_F64, 'cuda')
    acc = N.Accum()
    acc.slicer = ds.struct
    acc.partials = parts.data_ptr()
    acc.partials_len = parts.numel()
    acc.grid = G
    out = torch.empty(2, 3, S, dtype=torch.float64, device='cuda')
    N.call('phk_slice_sums', ctypes.byref(acc), out.data_ptr(),
           stream_handle())
    got = out.cpu().numpy()
    want = H.fold_columns(P)
    assert got.tobytes() == want.tobytes()
    # three shards of the columns, merged in rank order
    cuts = [0, 150, 300, G]
    pairs = np.stack([H.fold_columns(P[:, :, a:b])
                      for a, b in zip(cuts, cuts[1:])])
    dev_pairs = torch.from_numpy(pairs.copy()).cuda()
    cnt = torch.empty(S, dtype=torch.int32, device='cuda')
    mx = torch.empty(S, dtype=torch.float64, device='cuda')
    my = torch.empty(S, dtype=torch.float64, device='cuda')
    mom = torch.empty(3, S, dtype=torch.float64, device='cuda')
    N.call('phk_slice_merge', dev_pairs.data_ptr(), 3, S, cnt.data_ptr(),
           mx.data_ptr(), my.data_ptr(), mom.data_ptr(), stream_handle())
    n, hmx, hmy, hmom = H.finalize(H.merge_pairs(pairs))
    assert np.array_equal(cnt.cpu().numpy(), n)
    assert mx.cpu().numpy().tobytes() == hmx.tobytes()
    assert my.cpu().numpy().tobytes() == hmy.tobytes()
    assert mom.cpu().numpy().tobytes() == hmom.tobytes()
    exact = np.array([[math.fsum(P[q, s]) for s in range(S)]
                      for q in range(3)])
    assert H.merge_pairs(pairs).tobytes() == exact.tobytes()


class _ThreadShards(object):
    """In-process stand-in for a process group: shard threads exchange
    their tensors at a barrier, rank 0 first."""

    def __init__(self, rank, world, board, barrier):
        self.rank, self.world = rank, world
        self.board, self.barrier = board, barrier
        self.group = None

    def range(self, n):
        from pyheadtail_gb300.shards import shard_range
        return shard_range(n, self.rank, self.world)

    def all_gather(self, t):
        self.board[self.rank] = t.contiguous().clone()
        self.barrier.wait(timeout=120)
        out = torch.stack(list(self.board))
        self.barrier.wait(timeout=120)
        return out


def _spec(n):
    import cases as C
    return dict(beam=C.beam_params(n, 9), n_turns=N_TURNS, elements=[
        C.smooth_transverse(), C.rf(),
        C.wake(C.slicer(500), C.resonator(),
               C.resistive_wall(n_turns_wake=50))])


def _run(spec, coords, shards=None, counts_log=None):
    import gpu_cases as G
    from pyheadtail_gb300 import shards as SH
    beam = G.make_beam(spec['beam'], coords, precision='fp64')
    if shards is not None:
        SH.shard(beam, shards)
    els = [el for _, el in G.make_elements(spec, beam)]
    for t in range(N_TURNS):
        for el in els:
            el.track(beam)
        if counts_log is not None:
            ss = els[-1].slice_set_deque[0]
            counts_log.append((ss.n_macroparticles_per_slice.cpu().numpy(),
                               ss.mean_x.cpu().numpy(),
                               ss.mean_y.cpu().numpy()))
    beam.mean_x()
    return {k: getattr(beam, k).cpu().numpy().copy()
            for k in ('x', 'xp', 'y', 'yp', 'z', 'dp')}


def test_two_shards_follow_the_unsharded_bunch():
    from oracle import cases as OC
    n = 200001
    spec = _spec(n)
    coords = OC.make_beam(spec['beam']).coords()
    ref_log = []
    ref = _run(spec, coords, counts_log=ref_log)
    torch.cuda.synchronize()
    world = 2
    board = [None] * world
    barrier = threading.Barrier(world)
    results, logs, errors = [None] * world, [[] for _ in range(world)], []

    def worker(rank):
        try:
            sh = _ThreadShards(rank, world, board, barrier)
            a, b = sh.range(n)
            part = {k: v[a:b].copy() for k, v in coords.items()}
            results[rank] = _run(spec, part, shards=sh, counts_log=logs[rank])
            torch.cuda.synchronize()
        except Exception as exc:        # reported below
            errors.append(exc)
            barrier.abort()

    threads = [threading.Thread(target=worker, args=(r,)) for r in range(world)]
    for t in threads:
        t.start()
    for t in threads:
        t.join(timeout=600)
    assert not errors, errors
    for t_ref, t0, t1 in zip(ref_log, logs[0], logs[1]):
        for a, b in zip(t0, t1):
            assert a.tobytes() == b.tobytes()
        assert np.array_equal(t0[0], t_ref[0])
        for q in (1, 2):
            np.testing.assert_allclose(t0[q], t_ref[q], rtol=1e-13,
                                       atol=1e-13 * np.abs(t_ref[q]).max())
    for k, v in ref.items():
        got = np.concatenate([results[0][k], results[1][k]])
        rms = np.sqrt(np.mean(v**2))
        assert np.max(np.abs(got - v)) <= 1e-12 * rms, k


def test_sharded_bunch_refuses_bunch_dependent_cuts():
    import cases as C
    import gpu_cases as G
    from oracle import cases as OC
    from pyheadtail_gb300 import shards as SH
    bp = C.beam_params(1000, 1)
    beam = G.make_beam(bp, OC.make_beam(bp).coords())
    SH.shard(beam, SH.Shards())
    sl = G.make_slicer(C.slicer(50, z_cuts=None, n_sigma_z=3))
    with pytest.raises(NotImplementedError):
        sl.slice(beam)
