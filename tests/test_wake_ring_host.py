"""Host side of the multi-turn wake (no GPU): which wake-table rows are
recomputed from turn to turn, and when the tensor-core path's table
signature settles.

WakeField.track ages the stored slice sets by one revolution period each
turn (impedances/wakes.py:121-142 of the reference) and the kicks sample
their wake function for every stored turn (impedances/wake_kicks.py:
118-139).  With fixed cuts and energy, the samples of a lag never change
once that lag exists, so the table rows are rewritten only while the ring
fills, and a captured steady-state turn may keep the tables it was
captured with.  The turn loop
below performs WakeField.track's age and deque bookkeeping on host slice
sets."""
import types
from collections import deque

import numpy as np
import pytest

torch = pytest.importorskip('torch')

from scipy.constants import c  # noqa: E402

from pyheadtail_gb300.general.printers import SilentPrinter  # noqa: E402
from pyheadtail_gb300.impedances import wake_kicks as WK  # noqa: E402
from pyheadtail_gb300.impedances import wakes as W  # noqa: E402
from pyheadtail_gb300.particles.slicing import UniformBinSlicer  # noqa: E402

C_RING = 6911.5
RING = 12


def _kicks(sl):
    sources = [W.CircularResonator(10e6, 1e9, 1),
               W.CircularResistiveWall(0.02, C_RING, 5.8e7, 1e-12,
                                       n_turns_wake=RING)]
    kicks = []
    for s in sources:
        kicks += s.get_wake_kicks(sl)
    return kicks


def test_table_rows_are_written_only_while_the_ring_fills(monkeypatch):
    S = 40
    sl = UniformBinSlicer(S, z_cuts=(-0.69, 0.69),
                          warningprinter=SilentPrinter())
    kicks = _kicks(sl)
    assert sorted(k.n_turns_wake for k in kicks) == [1, 1, RING, RING]
    calls = []
    orig = WK.WakeKick._samples

    def counted(self, *a):
        calls.append(self)
        return orig(self, *a)
    monkeypatch.setattr(WK.WakeKick, '_samples', counted)

    beta = np.sqrt(1. - 1. / 27.7**2)
    slice_sets = deque([], maxlen=RING)
    ages = deque([], maxlen=RING)
    cpu = torch.device('cpu')
    prev = None
    changed = []
    for turn in range(3 * RING):
        for i in range(len(ages)):
            ages[i] += C_RING / (beta * c)
        zb = sl.z_bins(-0.69, 0.69)
        ss = types.SimpleNamespace(_times=sl.times(zb, beta), beta=beta)
        slice_sets.appendleft(ss)
        ages.appendleft(0.)
        del calls[:]
        for k in kicks:
            n_lags = k._sync_tables([s._times for s in slice_sets], ages,
                                    [s.beta for s in slice_sets], S, cpu)
            assert n_lags == min(turn + 1, k.n_turns_wake)
        # one new lag per multi-turn kick while the ring fills; the
        # single-turn kicks sample once; nothing afterwards
        want = (len(kicks) if turn == 0 else
                sum(k.n_turns_wake > 1 for k in kicks) if turn < RING else 0)
        assert len(calls) == want, turn
        sig = W._TensorWake.signature(kicks)
        changed.append(sig != prev)
        prev = sig
    assert changed == [True] * RING + [False] * (2 * RING)

    # every row holds the samples of its lag (the stored turn's times
    # shifted by its age), whatever turn wrote it
    times = [s._times for s in slice_sets]
    for k in kicks:
        for a in range(k.n_turns_wake):
            want = orig(k, times[0], times[a] + ages[a], beta)
            np.testing.assert_array_equal(k._table[a].numpy(), want.ravel())


def test_changed_cuts_rewrite_every_lag():
    S = 40
    sl = UniformBinSlicer(S, z_cuts=(-0.69, 0.69),
                          warningprinter=SilentPrinter())
    kick = [k for k in _kicks(sl) if k.n_turns_wake == RING][0]
    beta = np.sqrt(1. - 1. / 27.7**2)
    cpu = torch.device('cpu')
    t0 = sl.times(sl.z_bins(-0.69, 0.69), beta)
    ages = [i * C_RING / (beta * c) for i in range(RING)]
    kick._sync_tables([t0] * RING, ages, [beta] * RING, S, cpu)
    before = kick._table.clone()
    t1 = sl.times(sl.z_bins(-0.6, 0.6), beta)
    assert t1 is not t0
    kick._sync_tables([t1] * RING, ages, [beta] * RING, S, cpu)
    assert not any(torch.equal(before[a], kick._table[a])
                   for a in range(RING))
    # the same cuts again give the same cached times object: no rewrite
    assert sl.times(sl.z_bins(-0.6, 0.6), beta) is t1
