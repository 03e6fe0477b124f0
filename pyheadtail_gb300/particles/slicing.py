"""Uniform-bin slicing on the GPU.

Mirrors PyHEADTAIL's particles/slicing.py: ``clean_slices`` (:45-55),
``SliceSet`` (:58-317), ``Slicer`` (:320-529) and ``UniformBinSlicer``
(:532-615).  The slice index of every particle is the reference's
``int32(floor((z - z_cut_tail) / slice_width))`` bit for bit: the kernels
look it up in an exact lower-edge table built on the host from that very
formula (``pyheadtail_gb300._engine.exact_edges``), so no per-particle
division is needed.  Counts and the per-slice sums of x and y are
accumulated in the same pass that applies the pending element program.

Per-slice arrays of a SliceSet are torch CUDA tensors.  The particle index
array ``slice_index_of_particle`` is produced on demand by a slicing pass;
it can only be produced while the beam's z is still the one the SliceSet
was made from (SliceSets describe a past state), otherwise it raises.
"""
from abc import ABCMeta, abstractmethod
from functools import wraps

import numpy as np
import torch
from scipy.constants import c, e

from .. import _engine as E
from .. import _native as N
from ..general.element import Printing


def clean_slices(long_track_method):
    """Adds beam.clean_slices() to a track method that changes z."""
    @wraps(long_track_method)
    def cleaned(long_track_element, beam, *args, **kwargs):
        res = long_track_method(long_track_element, beam, *args, **kwargs)
        beam.clean_slices()
        return res
    return cleaned


class ModeIsUniformCharge(Exception):
    pass


class SliceSet(Printing):
    """Snapshot of a beam's longitudinal binning (slicing.py:58-317)."""

    def __init__(self, z_bins, mode, dslicer, beam, counts,
                 beam_parameters={}):
        self.age = 0
        self.z_bins = z_bins
        self.mode = mode
        self._dslicer = dslicer
        self._n_macroparticles_per_slice = counts
        self._beam = beam
        self._z_version = beam._engine.z_version
        self._slice_index_of_particle = None
        self._particles_within_cuts = None
        for k, v in beam_parameters.items():
            if hasattr(self, k):
                raise ValueError('SliceSet.' + k + ' already exists!')
            setattr(self, k, v)

    @property
    def z_cut_head(self):
        return self.z_bins[-1]

    @property
    def z_cut_tail(self):
        return self.z_bins[0]

    @property
    def z_centers(self):
        return self.z_bins[:-1] + 0.5 * (self.z_bins[1:] - self.z_bins[:-1])

    @property
    def n_slices(self):
        return len(self.z_bins) - 1

    @property
    def slice_widths(self):
        return np.diff(self.z_bins)

    @property
    def n_macroparticles_per_slice(self):
        return self._n_macroparticles_per_slice

    @property
    def charge_per_slice(self):
        return self.charge_per_mp * self.n_macroparticles_per_slice

    @property
    def slice_index_of_particle(self):
        if self._slice_index_of_particle is None:
            b = self._beam
            if b._engine.z_version != self._z_version:
                raise RuntimeError(
                    'slice_index_of_particle of a SliceSet must be read '
                    'before the beam is tracked further (the GPU SliceSet '
                    'keeps no copy of z); request it right after slicing')
            self._slice_index_of_particle = _index_pass(b, self._dslicer)
        return self._slice_index_of_particle

    @property
    def particles_within_cuts(self):
        if self._particles_within_cuts is None:
            idx = self.slice_index_of_particle
            self._particles_within_cuts = torch.nonzero(
                (idx < self.n_slices) & (idx >= 0)).flatten().to(torch.int32)
        return self._particles_within_cuts

    @property
    def particles_outside_cuts(self):
        idx = self.slice_index_of_particle
        return torch.nonzero(~((idx < self.n_slices) &
                               (idx >= 0))).flatten().to(torch.int32)

    @property
    def slice_positions(self):
        pos = torch.zeros(self.n_slices + 1, dtype=torch.int32,
                          device=self._n_macroparticles_per_slice.device)
        pos[1:] = torch.cumsum(self.n_macroparticles_per_slice, 0)
        return pos

    def particle_indices_of_slice(self, slice_index):
        p = self.particles_within_cuts
        return p[self.slice_index_of_particle[p] == slice_index]

    def convert_to_time(self, z):
        """slicing.py:303-307."""
        return z / (self.beta * c)

    def convert_to_particles(self, slice_array, empty_particles=None):
        out = (torch.zeros(self._beam.macroparticlenumber, dtype=torch.float64,
                           device=self._beam._device)
               if empty_particles is None else empty_particles.fill_(0))
        p = self.particles_within_cuts.long()
        s = self.slice_index_of_particle[p].long()
        out[p] = torch.as_tensor(slice_array, device=out.device,
                                 dtype=out.dtype)[s]
        return out


def _index_pass(beam, dslicer):
    """Slicing pass that writes the reference index of every particle."""
    idx = torch.empty(beam.macroparticlenumber, dtype=torch.int32,
                      device=beam._device)
    part, grid = beam._engine.workspace(dslicer.n_slices)
    beam._engine.slice_pass(E.AccumRequest(dslicer, part, grid, idx))
    return idx


class Slicer(Printing, metaclass=ABCMeta):
    """Factory of SliceSets (slicing.py:320-529)."""

    @property
    def config(self):
        return (self.mode, self.n_slices, self.n_sigma_z, self.z_cuts)

    @config.setter
    def config(self, value):
        self.mode, self.n_slices, self.n_sigma_z, self.z_cuts = value
        if self.z_cuts is not None and self.z_cuts[0] >= self.z_cuts[1]:
            self.warns('Slicer.config: z_cut_tail >= z_cut_head, this leads '
                       'to negative bin sizes and particle indices starting '
                       'at the head')

    def __hash__(self):
        return hash(self.config)

    def __eq__(self, other):
        return self.config == other.config

    def __ne__(self, other):
        return not self.__eq__(other)

    @staticmethod
    def extract_beam_parameters(beam):
        return dict(beta=beam.beta, gamma=beam.gamma, p0=beam.p0,
                    particlenumber_per_mp=beam.particlenumber_per_mp,
                    charge=beam.charge, charge_per_mp=beam.charge_per_mp,
                    mass=beam.mass, intensity=beam.intensity)

    def get_long_cuts(self, beam):
        """slicing.py:395-413."""
        if self.z_cuts is not None:
            return self.z_cuts
        elif self.n_sigma_z:
            tail = beam.mean_z() - self.n_sigma_z * beam.sigma_z()
            head = beam.mean_z() + self.n_sigma_z * beam.sigma_z()
        else:
            z = beam.z
            tail = float(torch.min(z))
            head = float(torch.max(z))
            head += abs(head) * 1e-15
        return tail, head

    @abstractmethod
    def slice(self, beam, *args, **kwargs):
        pass


class UniformBinSlicer(Slicer):
    """Uniform bins over the slicing region (slicing.py:532-615)."""

    def __init__(self, n_slices, n_sigma_z=None, z_cuts=None,
                 z_sample_points=None, *args, **kwargs):
        if n_sigma_z and (z_cuts or z_sample_points):
            raise ValueError('Argument n_sigma_z is incompatible with either '
                             'of z_cuts or z_sampling_points. Choose either '
                             'n_sigma_z or a combination of z_cuts and '
                             'z_sampling_points.')
        if z_sample_points is not None:
            self.warns('n_slices will be overridden to match given '
                       'combination of z_cuts and z_sampling_points.')
            n_slices, z_cuts = self._get_slicing_from_z_sample_points(
                z_sample_points, z_cuts)
        if not 1 <= n_slices <= N.PHK_MAX_SLICES:
            raise ValueError('n_slices must be in [1, %d]' % N.PHK_MAX_SLICES)
        self.config = ('uniform_bin', n_slices, n_sigma_z, z_cuts)
        self._dev_cache = {}
        self._times_cache = {}

    @staticmethod
    def _get_slicing_from_z_sample_points(z_sample_points, z_cuts=None):
        """slicing.py:556-597."""
        dz = np.diff(z_sample_points)[0]
        if not np.allclose(np.diff(z_sample_points) - dz, 1e-15):
            raise TypeError('Irregular sampling of wakes incompatible with '
                            'UniformBinSlicer. Check the sampling points.')
        n_slices = len(z_sample_points)
        aa, bb = z_sample_points[0] - dz / 2., z_sample_points[-1] + dz / 2.
        if z_cuts:
            if z_cuts[0] < aa:
                while z_cuts[0] < aa:
                    aa -= dz
                    n_slices += 1
            elif z_cuts[0] > aa:
                while z_cuts[0] > aa:
                    aa += dz
                    n_slices -= 1
            if z_cuts[1] < bb:
                while z_cuts[1] < bb:
                    bb -= dz
                    n_slices -= 1
            elif z_cuts[1] > bb:
                while z_cuts[1] > bb:
                    bb += dz
                    n_slices += 1
        return n_slices, (aa, bb)

    def device_slicer(self, tail, head, beam):
        key = (float(tail), float(head), beam._code, str(beam._device))
        ds = self._dev_cache.get(key)
        if ds is None:
            if len(self._dev_cache) > 8:
                self._dev_cache.clear()
            ds = E.DeviceSlicer(tail, head, self.n_slices, beam._code,
                                beam._device)
            self._dev_cache[key] = ds
        return ds

    def z_bins(self, tail, head):
        """slicing.py:605-608 (np.arange exactly as the reference)."""
        width = (head - tail) / float(self.n_slices)
        return np.arange(tail, head + 1e-7 * width, width, dtype=np.float64)

    def times(self, z_bins, beta):
        """convert_to_time(z_centers) with a cache, so that unchanged cuts and
        beta give the *same* array object (the wake tables key on it)."""
        key = (z_bins[0], z_bins[-1], len(z_bins), float(beta))
        t = self._times_cache.get(key)
        if t is None:
            if len(self._times_cache) > 64:
                self._times_cache.clear()
            zc = z_bins[:-1] + 0.5 * (z_bins[1:] - z_bins[:-1])
            t = zc / (beta * c)
            t.setflags(write=False)
            self._times_cache[key] = t
        return t

    def slice(self, beam, *args, **kwargs):
        """Slicer.slice (slicing.py:348-381) on the GPU."""
        stats = kwargs.get('statistics', None)
        ss = make_slice_set(self, beam, with_means=bool(stats))
        if stats:
            add_statistics(ss, beam, stats)
        return ss

    # -- statistics entry point kept for API parity (slicing.py:443-470)
    def add_statistics(self, sliceset, beam, statistics):
        add_statistics(sliceset, beam, statistics)


def make_slice_set(slicer, beam, with_means=False, moments_out=None):
    """Flush the beam's pending program with a fused slicing pass and wrap
    the per-slice results in a SliceSet."""
    tail, head = slicer.get_long_cuts(beam)
    ds = slicer.device_slicer(tail, head, beam)
    eng = beam._engine
    part, grid = eng.workspace(slicer.n_slices)
    acc = E.AccumRequest(ds, part, grid)
    eng.flush(acc)
    S = slicer.n_slices
    dev = beam._device
    counts = torch.empty(S, dtype=torch.int32, device=dev)
    mx = my = None
    if with_means or moments_out is not None:
        mx = torch.empty(S, dtype=torch.float64, device=dev)
        my = torch.empty(S, dtype=torch.float64, device=dev)
    a = acc.struct()
    N.call('phk_slice_finalize', __import__('ctypes').byref(a),
           counts.data_ptr(), 0 if mx is None else mx.data_ptr(),
           0 if my is None else my.data_ptr(),
           0 if moments_out is None else moments_out.data_ptr(),
           E.stream_handle())
    params = Slicer.extract_beam_parameters(beam)
    params['is_sorted'] = False
    ss = SliceSet(slicer.z_bins(tail, head), slicer.mode, ds, beam, counts,
                  beam_parameters=params)
    if mx is not None:
        ss.mean_x = mx
        ss.mean_y = my
    return ss


_STAT_COORDS = {'mean_x': 'x', 'mean_y': 'y', 'mean_z': 'z', 'mean_xp': 'xp',
                'mean_yp': 'yp', 'mean_dp': 'dp', 'sigma_x': 'x',
                'sigma_y': 'y', 'sigma_z': 'z', 'sigma_dp': 'dp'}
ALL_STATS = ['mean_x', 'mean_y', 'mean_z', 'mean_xp', 'mean_yp', 'mean_dp',
             'sigma_x', 'sigma_y', 'sigma_z', 'sigma_dp', 'epsn_x', 'epsn_y',
             'epsn_z', 'eff_epsn_x', 'eff_epsn_y']


def _slice_moments(ss, beam, names):
    """Per-slice means and centred second moments of up to three
    coordinates (two passes of phk_slice_moments; stats.pyx:235-425)."""
    import ctypes
    S = ss.n_slices
    dev = beam._device
    eng = beam._engine
    if not eng.idle:
        eng.flush()
    z = beam._c['z']
    qs = [beam._c[n] for n in names]
    arr = (ctypes.c_void_p * 3)(*[q.data_ptr() for q in qs] +
                                [None] * (3 - len(qs)))
    sums = torch.zeros(9, S, dtype=torch.float64, device=dev)
    counts = torch.zeros(S, dtype=torch.int32, device=dev)
    sl = ss._dslicer.struct
    N.call('phk_slice_moments', ctypes.byref(sl), z.data_ptr(),
           beam.macroparticlenumber, beam._code, arr, len(qs), 0, None,
           sums.data_ptr(), counts.data_ptr(), E.stream_handle())
    n = counts.double()
    means = torch.where(counts > 0, sums[:3] / n.clamp(min=1),
                        torch.zeros_like(sums[:3])).contiguous()
    N.call('phk_slice_moments', ctypes.byref(sl), z.data_ptr(),
           beam.macroparticlenumber, beam._code, arr, len(qs), 1,
           means.data_ptr(), sums.data_ptr(), None, E.stream_handle())
    big = counts > 1
    cov = torch.where(big, sums[3:] / (n - 1).clamp(min=1), sums[3:])
    return means, cov, counts


def add_statistics(ss, beam, statistics):
    """Slicer.add_statistics (slicing.py:443-529) for the GPU SliceSet."""
    if statistics is True:
        statistics = ALL_STATS
    for stat in statistics:
        if hasattr(ss, stat):
            continue
        if stat.startswith('mean_'):
            means, _, _ = _slice_moments(ss, beam, [_STAT_COORDS[stat]])
            setattr(ss, stat, means[0].clone())
        elif stat.startswith('sigma_'):
            _, cov, _ = _slice_moments(ss, beam, [_STAT_COORDS[stat]])
            setattr(ss, stat, torch.sqrt(cov[0]))
        elif stat in ('epsn_x', 'epsn_y', 'eff_epsn_x', 'eff_epsn_y',
                      'epsn_z'):
            if stat == 'epsn_z':
                names, disp, scale = ['z', 'dp'], False, None
            else:
                u = stat[-1]
                names = [u, u + 'p'] + ([] if stat.startswith('eff') else ['dp'])
                disp = not stat.startswith('eff')
            _, cov, counts = _slice_moments(ss, beam, names)
            # pairs: 0 (u,u) 1 (u,up) 2 (up,up) 3 (u,dp) 4 (up,dp) 5 (dp,dp)
            s11, s12, s22 = cov[0].clone(), cov[1].clone(), cov[2].clone()
            if disp:
                cdp2 = cov[5]
                ok = cdp2 != 0
                safe = torch.where(ok, cdp2, torch.ones_like(cdp2))
                s11 = torch.where(ok, s11 - cov[3] * cov[3] / safe, s11)
                s12 = torch.where(ok, s12 - cov[3] * cov[4] / safe, s12)
                s22 = torch.where(ok, s22 - cov[4] * cov[4] / safe, s22)
            em = torch.where(counts > 1, torch.sqrt(s11 * s22 - s12 * s12),
                             torch.zeros_like(s11))
            if stat == 'epsn_z':
                em = 4. * np.pi * em * beam.p0 / e
            else:
                em = em * beam.betagamma
            setattr(ss, stat, em)
        else:
            raise ValueError('unknown statistics ' + stat)
