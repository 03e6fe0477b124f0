"""Host logic of the batched form (no GPU): bunch offsets, the unit plan
that drives the persistent launch, the autotuner cache, and the host-side
validation of the batched C entry points, the batch storage and its
view check."""
import ctypes
import os

import numpy as np
import pytest
import torch

from pyheadtail_gb300 import _native as N
from pyheadtail_gb300 import batch as B


def test_bunch_offsets_are_aligned_and_disjoint():
    counts = [5, 0, 13, 4, 1, 1000003]
    off, total = B.bunch_offsets(counts)
    assert list(off % B.ALIGN) == [0] * len(counts)
    ends = off + np.array(counts)
    assert np.all(ends[:-1] <= off[1:])
    assert total >= ends[-1] and total % B.ALIGN == 0


@pytest.mark.parametrize('seed,grid,unit', [(0, 7, 64), (1, 304, 8192),
                                            (2, 1, 4), (3, 1000, 1024)])
def test_unit_plan_invariants(seed, grid, unit):
    rng = np.random.default_rng(seed)
    counts = np.round(10 ** rng.uniform(0, 4.5, 37)).astype(np.int64)
    counts[3] = 0
    off, total = B.bunch_offsets(counts)
    p = B.plan_units(off, counts, grid, unit)
    u, col, cf, bc = p['units'], p['column'], p['cta_first'], p['bunch_columns']
    # units tile every bunch exactly, start aligned, at most `unit` long
    for b in range(len(counts)):
        mine = u[u[:, 2] == b]
        got = sum(e - s for s, e, _ in mine)
        assert got == counts[b]
        if len(mine):
            assert mine[0, 0] == off[b] and mine[-1, 1] == off[b] + counts[b]
            assert np.all(mine[1:, 0] == mine[:-1, 1])
    assert np.all(u[:, 0] % B.ALIGN == 0)
    assert np.all(u[:, 1] - u[:, 0] <= unit) and np.all(u[:, 1] > u[:, 0])
    # CTA ranges: monotone, cover all units, balanced to within one unit
    assert cf[0] == 0 and cf[-1] == len(u) and np.all(np.diff(cf) >= 0)
    load = [int((u[cf[g]:cf[g + 1], 1] - u[cf[g]:cf[g + 1], 0]).sum())
            for g in range(grid)]
    assert max(load) <= int(counts.sum()) // grid + unit
    # columns: one per (CTA, bunch) run, numbered in unit order; bunch b's
    # columns are exactly bunch_columns[b] .. bunch_columns[b+1]-1
    assert p['n_columns'] == len(set(col.tolist())) or len(u) == 0
    for g in range(grid):
        r = range(cf[g], cf[g + 1])
        for i, j in zip(list(r)[:-1], list(r)[1:]):
            assert (col[i] == col[j]) == (u[i, 2] == u[j, 2])
    for b in range(len(counts)):
        cols = sorted(set(col[u[:, 2] == b].tolist()))
        assert cols == list(range(bc[b], bc[b + 1]))
    assert bc[-1] == p['n_columns'] or len(u) == 0


def test_unit_plan_rejects_unaligned_units():
    with pytest.raises(ValueError):
        B.plan_units([0], [10], 2, 6)


def test_autotune_cache_round_trip():
    path = os.path.join(os.path.dirname(B.default_cache_path()),
                        'test_cache_roundtrip.json')
    try:
        B.store_cache(path, {'k': {'threads': 128, 'unit_tiles': 4,
                                   'ctas_per_sm': 2}})
        assert B.load_cache(path)['k']['threads'] == 128
    finally:
        if os.path.exists(path):
            os.remove(path)


def test_candidates_cover_every_thread_count():
    cands = B.candidates(152, lambda t: 152 * (2048 // t // 2))
    assert {c['threads'] for c in cands} == set(B.THREADS)
    assert {c['unit_tiles'] for c in cands} == set(B.UNIT_TILES)
    assert all(c['ctas_per_sm'] >= 1 for c in cands)


def test_batch_struct_layout():
    assert ctypes.sizeof(N.Unit) == 24
    assert ctypes.sizeof(N.Batch) == 72
    assert N.Batch.units.offset == 24
    assert N.Batch.status.offset == 64


def test_batch_entry_points_validate_on_host():
    L = N.load(build_if_missing=False)
    assert L.phk_track_batch(None, None, None, None, None) == -1
    bt = N.Batch()
    bt.n_bunches, bt.n_units, bt.grid, bt.threads = 2, 1, 1, 100
    bt.units = bt.cta_first = bt.programs = 4096
    progs = (N.Program * 2)()
    bt.programs_host = ctypes.cast(progs, ctypes.POINTER(N.Program))
    c = N.Coords()
    assert L.phk_track_batch(ctypes.byref(bt), ctypes.byref(c), None, None,
                             None) == -4
    bt.threads = 256
    c.n, c.dtype = 8, N.PHK_F32
    for i, f in enumerate(('x', 'xp', 'y', 'yp', 'z', 'dp')):
        setattr(c, f, 4096 * (i + 1) + 4)          # 4-byte aligned only
    assert L.phk_track_batch(ctypes.byref(bt), ctypes.byref(c), None, None,
                             None) == -3
    for i, f in enumerate(('x', 'xp', 'y', 'yp', 'z', 'dp')):
        setattr(c, f, 4096 * (i + 1))
    progs[1].n_ops = 99
    assert L.phk_track_batch(ctypes.byref(bt), ctypes.byref(c), None, None,
                             None) == -2
    assert 'n_ops' in N.last_error()
    assert L.phk_wake_batch(4096, 3, 0, 2, None) == -2
    assert L.phk_wake_batch(None, 3, 10, 2, None) == -1
    assert L.phk_batch_finalize(None, 1, None, None, None, None, None, 0,
                                None) == -1
    assert L.phk_batch_max_grid(7, 256, 100, 2) == -4
    assert L.phk_batch_max_grid(0, 96, 100, 2) == -4


class _Engine(object):
    z_version = 0

    def flush(self):
        pass


class _Bunch(object):
    """The parts of Particles a BunchBatch touches, on CPU tensors."""

    def __init__(self, n, seed):
        g = torch.Generator().manual_seed(seed)
        self._c = {q: torch.randn(n, generator=g, dtype=torch.float64)
                   for q in ('x', 'xp', 'y', 'yp', 'z', 'dp')}
        self._code = N.PHK_F64
        self._device = torch.device('cpu')
        self._engine = _Engine()
        self.macroparticlenumber = n
        self._rebinds = 0


def test_batch_views_and_rebind_check():
    """A batch copies every bunch into one aligned storage and rebinds the
    bunches' arrays to views of it; check_views looks again only when a
    bunch's array was replaced (Particles counts that in _rebinds) and
    raises if it no longer lives in the batch."""
    from pyheadtail_gb300.batch import BunchBatch
    bunches = [_Bunch(n, i) for i, n in enumerate((1000, 37, 4096))]
    want = {id(b): {q: t.clone() for q, t in b._c.items()} for b in bunches}
    batch = BunchBatch(bunches)
    for b in bunches:
        for q, t in b._c.items():
            assert torch.equal(t, want[id(b)][q])
            o = int(batch.offsets[bunches.index(b)])
            assert t.data_ptr() == batch.storage[q][o:].data_ptr()
    batch.check_views()
    assert batch._rebinds_seen == [0, 0, 0]
    batch.check_views()                      # unchanged: no second look
    b = bunches[1]
    b._c['xp'] = b._c['xp'].clone()          # what Particles._set does
    b._rebinds += 1
    with pytest.raises(RuntimeError, match='bunch 1: coordinate xp'):
        batch.check_views()
