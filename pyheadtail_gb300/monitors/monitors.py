"""Monitors: BunchMonitor with a device-resident statistics ring, and
SliceMonitor / ParticleMonitor.

Mirrors ``BunchMonitor`` (monitors/monitors.py:39-186): the same
constructor (filename, n_steps, parameters_dict, write_buffer_every,
buffer_size, stats_to_store), ``dump(bunch)`` once per step, and a write
to file every ``write_buffer_every`` steps and at the last step.

The reference evaluates every statistic with its own pass and host sync at
each dump.  Here ``dump`` queues one ``phk_bunch_stats`` pass that appends a
record of the bunch's moment sums to a ring of ``buffer_size`` records on
the device (the device-side cursor picks the slot, so dumps need no host
sync and can sit inside a captured CUDA graph).  The records are read back
once per write and every statistic is evaluated on the host from them, with
the reference's formulas (pyheadtail_gb300.particles.statistics).
Attributes (``macroparticlenumber``) and statistics that are not moment
functions are taken on the host at dump time.

File format: HDF5 as the reference (group ``Bunch``, one dataset of
n_steps entries per statistic, parameters_dict as file attributes) when
h5py is importable; otherwise ``<filename>.npz`` with one array per
statistic and the parameters as a JSON string under ``__parameters__``.
"""
import json

import numpy as np
import torch
from scipy.constants import e

from ..general.element import Printing
from ..particles import statistics as S

DEFAULT_STATS = ['mean_x', 'mean_xp', 'mean_y', 'mean_yp', 'mean_z',
                 'mean_dp', 'sigma_x', 'sigma_y', 'sigma_z', 'sigma_dp',
                 'epsn_x', 'epsn_y', 'epsn_z', 'macroparticlenumber']

try:
    import h5py as _h5
except ImportError:
    _h5 = None


class Monitor(Printing):
    """Base of the monitors (monitors/monitors.py:25-37)."""

    def dump(self, bunch):
        raise NotImplementedError


class BunchMonitor(Monitor):
    """Bunch statistics per step, buffered on the device; see module."""

    def __init__(self, filename, n_steps, parameters_dict=None,
                 write_buffer_every=512, buffer_size=4096, *args, **kwargs):
        self.stats_to_store = list(kwargs.pop('stats_to_store',
                                              DEFAULT_STATS))
        self.filename = filename
        self.n_steps = int(n_steps)
        self.i_steps = 0
        self.buffer_size = int(buffer_size)
        self.write_buffer_every = int(write_buffer_every)
        if self.write_buffer_every > self.buffer_size:
            raise ValueError('write_buffer_every (%d) exceeds buffer_size '
                             '(%d): records would be overwritten on the '
                             'device before they are written'
                             % (self.write_buffer_every, self.buffer_size))
        self.parameters_dict = dict(parameters_dict or {})
        self._setup(self.stats_to_store, self.buffer_size)
        self._written = 0
        self._create_file_structure()

    # -- file
    def _create_file_structure(self):
        if _h5 is not None:
            with _h5.File(self.filename + '.h5', 'w') as f:
                for k, v in self.parameters_dict.items():
                    f.attrs[k] = v
                g = f.create_group('Bunch')
                for st in sorted(self.stats_to_store):
                    g.create_dataset(st, shape=(self.n_steps,),
                                     compression='gzip', compression_opts=9)
        else:
            self._arrays = {st: np.zeros(self.n_steps)
                            for st in self.stats_to_store}

    def _store(self, lo, hi, values):
        if _h5 is not None:
            with _h5.File(self.filename + '.h5', 'a') as f:
                for st in self.stats_to_store:
                    f['Bunch'][st][lo:hi] = values[st]
            return
        for st in self.stats_to_store:
            self._arrays[st][lo:hi] = values[st]
        np.savez(self.filename + '.npz',
                 __parameters__=np.array(json.dumps(self.parameters_dict,
                                                    default=str)),
                 **self._arrays)

    # -- stepping
    def _setup(self, stats, buffer_size):
        """The order and coordinates of the records these statistics need;
        the device ring is made at the first dump."""
        self.stats_to_store = list(stats)
        self.buffer_size = int(buffer_size)
        coords, order = (), 1
        for st in self.stats_to_store:
            if st in S.NEEDS:
                c, o = S.NEEDS[st]
                coords += c
                order = max(order, o)
        self._mask = S.mask_of(coords)
        self._order = order
        self._ring = None
        self._cursor = None
        self._host = {}        # step -> (betagamma, p0, host values)

    def _record(self, bunch, step):
        """Queue the statistics pass of ``step`` into the ring (no host
        sync, except for statistics that are not moment functions)."""
        if self._ring is None:
            dev = bunch._device
            self._ring = torch.zeros(self.buffer_size * S.RECORD_LEN,
                                     dtype=torch.float64, device=dev)
            self._cursor = torch.zeros(1, dtype=torch.int64, device=dev)
        if self._mask:
            bunch.launch_stats(self._ring, capacity=self.buffer_size,
                               cursor=self._cursor, order=self._order,
                               mask=self._mask)
        host = {}
        for st in self.stats_to_store:
            if st not in S.NEEDS:
                v = getattr(bunch, st)
                host[st] = v() if callable(v) else v
        self._host[step] = (bunch.betagamma, bunch.p0, host)

    def _evaluate(self, lo, hi):
        """The statistics of steps lo .. hi-1 from the ring (one read)."""
        rows = self._ring.view(self.buffer_size, S.RECORD_LEN).cpu().numpy()
        values = {st: np.zeros(hi - lo) for st in self.stats_to_store}
        for k, step in enumerate(range(lo, hi)):
            betagamma, p0, host = self._host.pop(step)
            rec = S.StatsRecord(rows[step % self.buffer_size], self._mask,
                                self._order)
            for st in self.stats_to_store:
                if st in S.NEEDS:
                    values[st][k] = rec.statistic(st, betagamma, p0, e)
                else:
                    values[st][k] = host[st]
        return values

    def dump(self, bunch):
        """Queue this step's statistics of ``bunch`` (no host sync, except
        for statistics that are not moment functions)."""
        if self.i_steps >= self.n_steps:
            raise IndexError('BunchMonitor: all %d steps are written'
                             % self.n_steps)
        self._record(bunch, self.i_steps)
        if ((self.i_steps + 1) % self.write_buffer_every == 0 or
                self.i_steps + 1 == self.n_steps):
            self._write_buffer_to_file()
        self.i_steps += 1

    def _write_buffer_to_file(self):
        lo, hi = self._written, self.i_steps + 1
        self._store(lo, hi, self._evaluate(lo, hi))
        self._written = hi


DEFAULT_SLICE_STATS = ['mean_x', 'mean_xp', 'mean_y', 'mean_yp', 'mean_z',
                       'mean_dp', 'sigma_x', 'sigma_y', 'sigma_z', 'sigma_dp',
                       'epsn_x', 'epsn_y', 'epsn_z',
                       'n_macroparticles_per_slice']


class SliceMonitor(Monitor):
    """Bunch and per-slice statistics per step (monitors/monitors.py:
    189-364): the same constructor (filename, n_steps, slicer,
    parameters_dict, write_buffer_every, buffer_size, bunch_stats_to_store,
    slice_stats_to_store) and file layout (groups ``Bunch`` with one
    dataset of n_steps entries per statistic, ``Slices`` with one dataset
    of n_slices x n_steps).  The slice statistics of a dump stay on the
    device (a [statistic][slice][buffer_size] tensor) and the bunch
    statistics go to a record ring as in BunchMonitor; the host reads both
    once per write.  The slicer needs fixed cuts (the dataset shape)."""

    def __init__(self, filename, n_steps, slicer, parameters_dict=None,
                 write_buffer_every=512, buffer_size=4096, *args, **kwargs):
        self.bunch_stats_to_store = list(kwargs.pop('bunch_stats_to_store',
                                                    DEFAULT_STATS))
        self.slice_stats_to_store = list(kwargs.pop('slice_stats_to_store',
                                                    DEFAULT_SLICE_STATS))
        self.filename = filename
        self.n_steps = int(n_steps)
        self.i_steps = 0
        self.slicer = slicer
        self.buffer_size = int(buffer_size)
        self.write_buffer_every = int(write_buffer_every)
        if self.write_buffer_every > self.buffer_size:
            raise ValueError('write_buffer_every (%d) exceeds buffer_size (%d)'
                             % (self.write_buffer_every, self.buffer_size))
        self.parameters_dict = dict(parameters_dict or {})
        # the bunch statistics ride on a BunchMonitor that never writes
        self._bunch = BunchMonitor.__new__(BunchMonitor)
        BunchMonitor._setup(self._bunch, self.bunch_stats_to_store,
                            self.buffer_size)
        self._slices = None
        self._written = 0
        S = slicer.n_slices
        self._arrays = {('Bunch', st): np.zeros(self.n_steps)
                        for st in self.bunch_stats_to_store}
        self._arrays.update({('Slices', st): np.zeros((S, self.n_steps))
                             for st in self.slice_stats_to_store})
        _create_file(self.filename, self.parameters_dict, self._arrays)

    def dump(self, bunch):
        """Slice the bunch with all statistics (monitors.py:308-325) and
        queue this step's values on the device."""
        if self.i_steps >= self.n_steps:
            raise IndexError('SliceMonitor: all %d steps are written'
                             % self.n_steps)
        slice_set = bunch.get_slices(self.slicer, statistics=True)
        slot = self.i_steps % self.buffer_size
        if self._slices is None:
            self._slices = torch.zeros(
                len(self.slice_stats_to_store), self.slicer.n_slices,
                self.buffer_size, dtype=torch.float64, device=bunch._device)
        for k, st in enumerate(self.slice_stats_to_store):
            v = getattr(slice_set, st)
            self._slices[k, :, slot] = torch.as_tensor(
                v, device=bunch._device).to(torch.float64)
        self._bunch._record(bunch, self.i_steps)
        if ((self.i_steps + 1) % self.write_buffer_every == 0 or
                self.i_steps + 1 == self.n_steps):
            self._write_buffer_to_file()
        self.i_steps += 1

    def _write_buffer_to_file(self):
        lo, hi = self._written, self.i_steps + 1
        steps = np.arange(lo, hi)
        bunch_vals = self._bunch._evaluate(lo, hi)
        sl = self._slices.cpu().numpy()
        for st in self.bunch_stats_to_store:
            self._arrays[('Bunch', st)][lo:hi] = bunch_vals[st]
        for k, st in enumerate(self.slice_stats_to_store):
            self._arrays[('Slices', st)][:, lo:hi] = \
                sl[k][:, steps % self.buffer_size]
        _store(self.filename, self.parameters_dict, self._arrays, lo, hi)
        self._written = hi


class ParticleMonitor(Monitor):
    """Coordinates of every stride-th macroparticle per dump
    (monitors/monitors.py:367-470): HDF5 group ``Step#<i>`` per dump in
    ``<filename>.h5part`` when h5py is present, else ``<filename>.Step#<i>
    .npz``; optional extra arrays per dump (``arrays_dict``)."""

    def __init__(self, filename, stride=1, parameters_dict=None, *args,
                 **kwargs):
        self.quantities_to_store = list(kwargs.pop(
            'quantities_to_store', ['x', 'xp', 'y', 'yp', 'z', 'dp', 'id']))
        self.filename = filename
        self.stride = int(stride)
        self.i_steps = 0
        self.parameters_dict = dict(parameters_dict or {})
        if _h5 is not None:
            with _h5.File(self.filename + '.h5part', 'w') as f:
                for k, v in self.parameters_dict.items():
                    f.attrs[k] = v

    def dump(self, bunch, arrays_dict=None):
        """monitors.py:434-470: the quantities (device arrays strided on the
        device, then read back) and the extra arrays of this dump."""
        values = {}
        for q in self.quantities_to_store:
            v = getattr(bunch, q)
            v = v[::self.stride] if hasattr(v, 'cpu') else v
            values[q] = v.cpu().numpy() if hasattr(v, 'cpu') else np.asarray(v)
        if arrays_dict is not None:
            for k, v in arrays_dict.items():
                v = v.cpu().numpy() if hasattr(v, 'cpu') else np.asarray(v)
                values[k] = v[::self.stride]
        name = 'Step#%d' % self.i_steps
        if _h5 is not None:
            with _h5.File(self.filename + '.h5part', 'a') as f:
                g = f.create_group(name)
                for k, v in values.items():
                    g.create_dataset(k, data=v, compression='gzip',
                                     compression_opts=9)
        else:
            np.savez(self.filename + '.' + name + '.npz', **values)
        self.i_steps += 1


def _create_file(filename, parameters_dict, arrays):
    """HDF5 file with groups and datasets of the given shapes (or nothing
    to create for the .npz fallback, which is written whole)."""
    if _h5 is None:
        return
    with _h5.File(filename + '.h5', 'w') as f:
        for k, v in parameters_dict.items():
            f.attrs[k] = v
        for (group, st), a in sorted(arrays.items()):
            g = f.require_group(group)
            g.create_dataset(st, shape=a.shape, compression='gzip',
                             compression_opts=9)


def _store(filename, parameters_dict, arrays, lo, hi):
    if _h5 is not None:
        with _h5.File(filename + '.h5', 'a') as f:
            for (group, st), a in arrays.items():
                f[group][st][..., lo:hi] = a[..., lo:hi]
        return
    np.savez(filename + '.npz',
             __parameters__=np.array(json.dumps(parameters_dict, default=str)),
             **{'%s/%s' % k: a for k, a in arrays.items()})
