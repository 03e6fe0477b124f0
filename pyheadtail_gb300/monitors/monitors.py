"""BunchMonitor with a device-resident statistics ring.

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
    def dump(self, bunch):
        """Queue this step's statistics of ``bunch`` (no host sync, except
        for statistics that are not moment functions)."""
        if self.i_steps >= self.n_steps:
            raise IndexError('BunchMonitor: all %d steps are written'
                             % self.n_steps)
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
        self._host[self.i_steps] = (bunch.betagamma, bunch.p0, host)
        if ((self.i_steps + 1) % self.write_buffer_every == 0 or
                self.i_steps + 1 == self.n_steps):
            self._write_buffer_to_file()
        self.i_steps += 1

    def _write_buffer_to_file(self):
        lo, hi = self._written, self.i_steps + 1
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
        self._store(lo, hi, values)
        self._written = hi
