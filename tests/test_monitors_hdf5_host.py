"""The HDF5 files of the monitors (no GPU, no h5py): this repository's
BunchMonitor, SliceMonitor and ParticleMonitor write through an in-memory
h5py stand-in (tests/fake_h5py.py) the same files as the reference's
monitors (monitors/monitors.py:39-470) -- attributes, groups, dataset
names, shapes, dtypes, compression and contents -- recorded by
tests/golden/make_golden_monitors.py from the reference itself.

The bunch statistics are the cases' values (monitor_cases.py); the device
passes that produce them on a GPU are replaced by those values, so what is
checked here is the file layout and the write schedule."""
import json
import os

import numpy as np
import pytest

torch = pytest.importorskip('torch')

import fake_h5py  # noqa: E402
import monitor_cases as MC  # noqa: E402
from pyheadtail_gb300.monitors import monitors as M  # noqa: E402

GOLDEN = os.path.join(os.path.dirname(__file__), 'golden', 'monitors',
                      'layout.npz')


def _golden(fname):
    with np.load(GOLDEN) as f:
        meta = json.loads(str(f['__meta__']))[fname]
        data = {k.split('::', 2)[2]: f[k] for k in f.files
                if k.startswith('data::%s::' % fname)}
    return meta, data


def _compare(fname):
    meta, data = _golden(fname)
    got = fake_h5py.snapshot(fname)
    assert got['attrs'] == meta['attrs']
    assert got['groups'] == meta['groups']
    assert sorted(got['datasets']) == sorted(meta['datasets'])
    for path, want in meta['datasets'].items():
        g = got['datasets'][path]
        for key in ('shape', 'dtype', 'compression', 'compression_opts'):
            assert g[key] == want[key], (fname, path, key)
        np.testing.assert_array_equal(g['data'], data[path],
                                      err_msg='%s %s' % (fname, path))


@pytest.fixture
def h5(monkeypatch, tmp_path):
    fake_h5py.reset()
    monkeypatch.setattr(M, '_h5', fake_h5py)
    monkeypatch.chdir(tmp_path)
    yield fake_h5py
    fake_h5py.reset()


def _bunch_values(stats):
    def evaluate(lo, hi):
        return {st: np.array([MC.bunch_value(st, s) for s in range(lo, hi)],
                             dtype=np.float64) for st in stats}
    return evaluate


def test_bunch_monitor_file(h5):
    r = MC.BUNCH_RUN
    mon = M.BunchMonitor('bunch', r['n_steps'], dict(MC.PARAMETERS),
                         write_buffer_every=r['write_buffer_every'],
                         buffer_size=r['buffer_size'])
    assert mon.stats_to_store == MC.BUNCH_STATS
    writes = []
    mon._record = lambda bunch, step: None
    evaluate = _bunch_values(mon.stats_to_store)

    def logged(lo, hi):
        writes.append((lo, hi))
        return evaluate(lo, hi)
    mon._evaluate = logged
    for _ in range(r['n_steps']):
        mon.dump(None)
    # every third step and the last one
    assert writes == [(0, 3), (3, 6), (6, 9), (9, 10)]
    _compare('bunch.h5')
    with pytest.raises(IndexError):
        mon.dump(None)


class _SlicedBunch(object):
    """The slice statistics of the current step; the bunch statistics go
    through the BunchMonitor ring, replaced by the cases' values."""
    _device = torch.device('cpu')

    def __init__(self, n_slices):
        self.step = 0
        self.n_slices = n_slices

    def get_slices(self, slicer, statistics=None):
        ss = type('SliceSetValues', (), {})()
        for st in MC.SLICE_STATS:
            setattr(ss, st, MC.slice_value(st, self.step, self.n_slices))
        return ss


def test_slice_monitor_file(h5):
    r = MC.SLICE_RUN
    slicer = type('SlicerShape', (), {'n_slices': r['n_slices']})()
    mon = M.SliceMonitor('slices', r['n_steps'], slicer, dict(MC.PARAMETERS),
                         write_buffer_every=r['write_buffer_every'],
                         buffer_size=r['buffer_size'])
    assert mon.bunch_stats_to_store == MC.BUNCH_STATS
    assert mon.slice_stats_to_store == MC.SLICE_STATS
    mon._bunch._record = lambda bunch, step: None
    mon._bunch._evaluate = _bunch_values(mon.bunch_stats_to_store)
    bunch = _SlicedBunch(r['n_slices'])
    for step in range(r['n_steps']):
        bunch.step = step
        mon.dump(bunch)
    _compare('slices.h5')


class _CoordBunch(object):
    def __init__(self, step, n):
        arrays, self.extra = MC.particle_arrays(step, n)
        for k, v in arrays.items():
            setattr(self, k, torch.from_numpy(v))   # device arrays


def test_particle_monitor_file(h5):
    r = MC.PARTICLE_RUN
    mon = M.ParticleMonitor('particles', stride=r['stride'],
                            parameters_dict=dict(MC.PARAMETERS))
    assert mon.quantities_to_store == MC.COORDS
    for step in range(r['n_dumps']):
        b = _CoordBunch(step, r['n'])
        mon.dump(b, arrays_dict=b.extra)
    _compare('particles.h5part')


def test_monitor_files_without_h5py(monkeypatch, tmp_path):
    """Without h5py: one .npz per BunchMonitor with the same statistics and
    the parameters as JSON."""
    monkeypatch.setattr(M, '_h5', None)
    monkeypatch.chdir(tmp_path)
    r = MC.BUNCH_RUN
    mon = M.BunchMonitor('bunch', r['n_steps'], dict(MC.PARAMETERS),
                         write_buffer_every=r['write_buffer_every'],
                         buffer_size=r['buffer_size'])
    mon._record = lambda bunch, step: None
    mon._evaluate = _bunch_values(mon.stats_to_store)
    for _ in range(r['n_steps']):
        mon.dump(None)
    meta, data = _golden('bunch.h5')
    with np.load('bunch.npz') as f:
        assert json.loads(str(f['__parameters__'])) == meta['attrs']
        for st in MC.BUNCH_STATS:
            # the .npz keeps FP64; the HDF5 file holds float32 as h5py's
            # default dataset type
            np.testing.assert_array_equal(
                f[st].astype(np.float32), data['Bunch/' + st])
