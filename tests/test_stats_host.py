"""Host side of the bunch statistics (no GPU).

* The statistics that pyheadtail_gb300.particles.statistics derives from a
  record of moment sums reproduce the reference's own values (the
  ``bunch_statistics`` fixture, made by running PyHEADTAIL) from the
  fixture's coordinates, for all 26 statistics of Particles.
* Edge cases of the formulas: n = 0, 1, 2, constant dp.
* BunchMonitor's ring / cursor / write logic, driven by a CPU stand-in
  bunch that writes the record phk_bunch_stats would write; SliceMonitor's
  device buffers and file layout, and ParticleMonitor's strided dumps, with
  CPU stand-ins of the bunch and its slice set.
"""
import json
import os

import numpy as np
import pytest
from scipy.constants import e

from oracle import turn_loop as T

torch = pytest.importorskip('torch')

from pyheadtail_gb300.particles import statistics as S  # noqa: E402

GOLDEN = os.path.join(os.path.dirname(__file__), 'golden')
COORDS = S.COORDS


def host_record(coords):
    """The record phk_bunch_stats writes, summed on the host in FP64."""
    d = [np.asarray(coords[q], dtype=np.float64) for q in COORDS]
    n = d[0].shape[0]
    r = np.zeros(S.RECORD_LEN)
    r[0] = n
    if n == 0:
        return r
    dd = [u - u[0] for u in d]
    for i in range(6):
        r[1 + i] = d[i][0]
        r[7 + i] = np.sum(dd[i])
    p = 13
    for a in range(6):
        for b in range(a, 6):
            r[p] = np.sum(dd[a] * dd[b])
            p += 1
    return r


def fixture():
    with np.load(os.path.join(GOLDEN, 'bunch_statistics.npz')) as f:
        return {k: f[k] for k in f.files}


def test_needs_cover_every_statistic():
    import cases as C
    assert sorted(S.NEEDS) == sorted(C.BUNCH_STATS)


@pytest.mark.parametrize('turn', [0, 2])
def test_record_statistics_match_reference(turn):
    g = fixture()
    spec = json.loads(str(g['spec']))
    coords = {q: g['t%d_%s' % (turn, q)] for q in COORDS}
    rec = S.StatsRecord(host_record(coords))
    gamma = float(g['t%d_gamma' % turn])
    betagamma = np.sqrt(gamma**2 - 1)
    p0 = float(g['t%d_p0' % turn])
    for name in spec['record_bunch_stats']:
        v = float(g['t%d_bs_%s' % (turn, name)])
        got = rec.statistic(name, betagamma, p0, e)
        scale = abs(v)
        if name.startswith('mean_'):
            scale = max(scale, float(g['t%d_bs_sigma_%s' % (turn, name[5:])]))
        assert abs(got - v) <= 1e-12 * scale, (name, got, v)


def test_small_and_degenerate_bunches():
    rng = np.random.RandomState(5)
    for n in (0, 1, 2, 3):
        c = {q: rng.normal(size=n) for q in COORDS}
        rec = S.StatsRecord(host_record(c))
        if n == 0:
            assert np.isnan(rec.mean('x'))
        else:
            assert abs(rec.mean('x') - np.mean(c['x'])) <= 1e-15
        if n < 2:
            assert rec.cov('x', 'xp') == 0.
            assert rec.std('z') == 0.
        else:
            assert abs(rec.cov('x', 'xp') - T.cov_shifted(c['x'], c['xp'])) \
                <= 1e-15
    # constant dp: the dispersive terms drop out (stats.pyx:103-104)
    c = {q: rng.normal(size=50) for q in COORDS}
    c['dp'] = np.full(50, 1e-3)
    rec = S.StatsRecord(host_record(c))
    assert rec.cov('dp', 'dp') == 0.
    assert abs(rec.emittance('x', 'xp', 'dp') -
               T.emittance(c['x'], c['xp'], c['dp'])) <= 1e-14
    assert abs(rec.dispersion('x') - T.dispersion(c['x'], c['dp'])) <= 1e-12


class _HostBunch(object):
    """Stand-in with the interface BunchMonitor uses; writes the records
    that phk_bunch_stats would write into a CPU ring."""

    def __init__(self, coords, gamma=27.7):
        self.c = coords
        self._device = torch.device('cpu')
        self.macroparticlenumber = len(coords['x'])
        self.betagamma = np.sqrt(gamma**2 - 1)
        self.p0 = 1e-17

    def launch_stats(self, records, capacity=1, cursor=None, order=2,
                     mask=0x3f):
        c = int(cursor[0]) if cursor is not None else 0
        r = host_record(self.c)
        slot = c % capacity
        records[slot * S.RECORD_LEN:(slot + 1) * S.RECORD_LEN] = \
            torch.from_numpy(r)
        if cursor is not None:
            cursor[0] = c + 1


def test_bunch_monitor_ring_and_writes(tmp_path):
    from pyheadtail_gb300.monitors.monitors import BunchMonitor
    rng = np.random.RandomState(9)
    fn = str(tmp_path / 'bm')
    n_steps = 11
    mon = BunchMonitor(fn, n_steps, {'turns': n_steps}, write_buffer_every=3,
                       buffer_size=4)
    want = {st: [] for st in mon.stats_to_store}
    for step in range(n_steps):
        c = {q: rng.normal(size=200) * (1 + step) for q in COORDS}
        b = _HostBunch(c)
        mon.dump(b)
        ob = T.Beam(c, 1., e, 1.67e-27, 100., 27.7)
        for st in mon.stats_to_store:
            if st == 'macroparticlenumber':
                want[st].append(200)
            elif st == 'epsn_z':
                # the oracle's p0 is its own; compare the emittance part
                want[st].append(4 * np.pi * T.emittance(c['z'], c['dp'], None)
                                * b.p0 / e)
            elif st.startswith('epsn_'):
                want[st].append(getattr(ob, st)() / ob.betagamma * b.betagamma)
            else:
                want[st].append(getattr(ob, st)())
    if os.path.exists(fn + '.h5'):
        pytest.skip('h5py present: file layout checked by the reference')
    with np.load(fn + '.npz') as f:
        assert json.loads(str(f['__parameters__'])) == {'turns': n_steps}
        for st in mon.stats_to_store:
            np.testing.assert_allclose(f[st], want[st], rtol=1e-12,
                                       atol=1e-30, err_msg=st)
    with pytest.raises(IndexError):
        mon.dump(b)
    with pytest.raises(ValueError):
        BunchMonitor(fn, 4, write_buffer_every=8, buffer_size=4)


class _HostSliceSet(object):
    def __init__(self, c, n_slices):
        z = c['z']
        edges = np.linspace(-1., 1., n_slices + 1)
        idx = np.searchsorted(edges, z, side='right') - 1
        inside = (idx >= 0) & (idx < n_slices)
        self.n_macroparticles_per_slice = torch.from_numpy(
            np.bincount(idx[inside], minlength=n_slices).astype(np.int32))
        for st in ('mean_x', 'mean_xp', 'mean_y', 'mean_yp', 'mean_z',
                   'mean_dp', 'sigma_x', 'sigma_y', 'sigma_z', 'sigma_dp',
                   'epsn_x', 'epsn_y', 'epsn_z'):
            setattr(self, st, torch.from_numpy(
                np.arange(n_slices, dtype=np.float64) * (1 + len(st)) +
                float(np.sum(z))))


class _HostSlicedBunch(_HostBunch):
    def get_slices(self, slicer, statistics=None):
        return _HostSliceSet(self.c, slicer.n_slices)


class _Slicer(object):
    n_slices = 7


def test_slice_monitor_writes(tmp_path):
    from pyheadtail_gb300.monitors.monitors import SliceMonitor
    rng = np.random.RandomState(2)
    fn = str(tmp_path / 'sm')
    n_steps = 9
    mon = SliceMonitor(fn, n_steps, _Slicer(), {'a': 1},
                       write_buffer_every=4, buffer_size=4)
    want_b, want_s = [], []
    for step in range(n_steps):
        c = {q: rng.normal(size=300) * 0.3 for q in COORDS}
        b = _HostSlicedBunch(c)
        mon.dump(b)
        want_b.append(np.mean(c['x']))
        want_s.append(_HostSliceSet(c, 7).n_macroparticles_per_slice.numpy())
    if os.path.exists(fn + '.h5'):
        pytest.skip('h5py present')
    with np.load(fn + '.npz') as f:
        np.testing.assert_allclose(f['Bunch/mean_x'], want_b, rtol=1e-12)
        np.testing.assert_array_equal(
            f['Slices/n_macroparticles_per_slice'], np.array(want_s).T)
        assert f['Slices/mean_x'].shape == (7, n_steps)


class _ParticleBunch(object):
    def __init__(self, n):
        for q in COORDS:
            setattr(self, q, torch.arange(n, dtype=torch.float64) * (1 + len(q)))
        self.id = torch.arange(1, n + 1, dtype=torch.int32)


def test_particle_monitor_writes(tmp_path):
    from pyheadtail_gb300.monitors.monitors import ParticleMonitor
    fn = str(tmp_path / 'pm')
    mon = ParticleMonitor(fn, stride=3)
    b = _ParticleBunch(20)
    mon.dump(b)
    mon.dump(b, arrays_dict={'extra': np.arange(20)})
    if os.path.exists(fn + '.h5part'):
        pytest.skip('h5py present')
    with np.load(fn + '.Step#1.npz') as f:
        np.testing.assert_array_equal(f['id'], np.arange(1, 21)[::3])
        np.testing.assert_array_equal(f['x'], np.arange(20)[::3] * 2.)
        np.testing.assert_array_equal(f['extra'], np.arange(20)[::3])
