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
from functools import partial, wraps

import numpy as np
import torch
from scipy import interpolate, ndimage
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


def make_int32(array):
    """slicing.py:29-30."""
    return array.astype(np.int32)


class ModeIsUniformCharge(Exception):
    """slicing.py:33-37."""

    def __init__(self, message):
        self.message = message

    def __str__(self):
        return self.message


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
        self._particle_indices_by_slice = None
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
    def smoothing_sigma(self):
        """slicing.py:133-134."""
        return 0.02 * self.n_slices

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
            idx = _index_pass(b, self._dslicer)
            if self.mode == 'uniform_charge':
                # the reference marks particles outside the cuts with -1
                # (slicing.py:668-673)
                idx = torch.where((idx >= 0) & (idx < self.n_slices), idx,
                                  torch.full_like(idx, -1))
            self._slice_index_of_particle = idx
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

    @property
    def particles_within_cuts_slice(self):
        """slicing.py:187-197.  The particles are never reordered by the
        slicing here (is_sorted is False), so this is particles_within_cuts
        as on the reference's CPU path."""
        if getattr(self, 'is_sorted', False):
            return slice(self.pidx_begin, self.pidx_end, 1)
        return self.particles_within_cuts

    @property
    def pidx_begin(self):
        """Index of the first particle within the cuts (slicing.py:199-204)."""
        return int(self.particles_within_cuts[0])

    @property
    def pidx_end(self):
        """Index after the last particle within the cuts (:206-211)."""
        return int(self.particles_within_cuts[-1]) + 1

    @property
    def particle_indices_by_slice(self):
        """Particle indices within the cuts grouped by slice, ascending
        inside a slice (the counting sort of slicing.py:214-227): a stable
        sort of particles_within_cuts by slice index."""
        if self._particle_indices_by_slice is None:
            p = self.particles_within_cuts
            s = self.slice_index_of_particle[p.long()]
            order = torch.sort(s, stable=True)[1]
            self._particle_indices_by_slice = p[order]
        return self._particle_indices_by_slice

    def particle_indices_of_slice(self, slice_index):
        p = self.particles_within_cuts
        return p[self.slice_index_of_particle[p] == slice_index]

    # -- line density (slicing.py:229-292), on the host from the counts
    def _counts_host(self):
        n = self.n_macroparticles_per_slice
        n = n.cpu().numpy() if torch.is_tensor(n) else np.asarray(n)
        return n.astype(np.int32)

    def lambda_bins(self, sigma=None, smoothen=True):
        """Line charge density per bin (slicing.py:229-237)."""
        if sigma is None:
            sigma = self.smoothing_sigma
        lambda_of_bins = self._counts_host() * self.charge_per_mp
        if smoothen:
            lambda_of_bins = ndimage.gaussian_filter1d(
                lambda_of_bins, sigma=sigma, mode='nearest')
        return lambda_of_bins

    def lambda_prime_bins(self, sigma=None, smoothen_before=True,
                          smoothen_after=True):
        """Derivative of the line charge density per bin, Gaussian-smoothed
        (slicing.py:239-268); the smoothing before the gradient acts on the
        int32 counts, as the reference's does."""
        if self.mode == 'uniform_charge':
            raise ModeIsUniformCharge('The derivative is zero up to '
                                      'numerical fluctuations because the '
                                      'charges have been distributed '
                                      'uniformly across the slices.')
        if sigma is None:
            sigma = self.smoothing_sigma
        smoothen = partial(ndimage.gaussian_filter1d, sigma=sigma,
                           mode='nearest')
        line_density = self._counts_host()
        if smoothen_before:
            line_density = smoothen(line_density)
        mp_density_derivative = np.gradient(line_density,
                                            self.slice_widths[0])
        if smoothen_after:
            mp_density_derivative = smoothen(mp_density_derivative)
        return mp_density_derivative * self.charge_per_mp

    def lambda_z(self, z=None, sigma=None, smoothen=True):
        """Line charge density along z (slicing.py:270-281)."""
        lambda_along_bins = (self.lambda_bins(sigma, smoothen)
                             / self.slice_widths)
        if z is None:
            return lambda_along_bins
        tck = interpolate.splrep(self.z_centers, lambda_along_bins, s=0)
        return interpolate.splev(z, tck, der=0, ext=1)

    def lambda_prime_z(self, z, sigma=None, smoothen_before=True,
                       smoothen_after=True):
        """Derivative of the line charge density along z (:283-292)."""
        lp_along_bins = self.lambda_prime_bins(
            sigma, smoothen_before, smoothen_after) / self.slice_widths
        tck = interpolate.splrep(self.z_centers, lp_along_bins, s=0)
        return interpolate.splev(z, tck, der=0, ext=1)

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

    def update_slices(self, beam):
        """Removed from the reference's interface (slicing.py:428-436)."""
        raise RuntimeError('update_slices(beam) no longer exists. '
                           'Instead, remove all previously recorded SliceSet'
                           'objects in the beam via beam.clean_slices() '
                           'when the longitudinal state of the beam is '
                           'changed. Concretely: replace '
                           'slices.update_slices(beam) by '
                           'beam.clean_slices().The SliceSet objects should '
                           'be retrieved via beam.get_slices(Slicer) '
                           '*only*. In this way the beam can memorize '
                           'previously created slice snapshots. This '
                           'minimises computation time.')

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

    def compute_sliceset_kwargs(self, beam):
        """The SliceSet arguments of the beam's current state
        (slicing.py:340-346, 599-615, 636-686): z_bins, the slice index of
        every particle, the mode and the counts per slice."""
        ss = make_slice_set(self, beam)
        return dict(z_bins=ss.z_bins,
                    slice_index_of_particle=ss.slice_index_of_particle,
                    mode=ss.mode,
                    n_macroparticles_per_slice=ss.n_macroparticles_per_slice)


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


def charge_bins_for(n):
    """Coarse bins of the order-statistics histogram: about 64 particles per
    bin, 256 to 8192 bins."""
    return int(min(8192, max(256, 1 << int(np.ceil(np.log2(max(n, 2) / 64.))))))


def charge_ranks(n, n_cut_tail, n_cut_head, n_slices):
    """Particles per slice and the ranks (inside the cuts) of the order
    statistics a uniform-charge slicing needs (slicing.py:645-665):
    z_sorted[first - 1] and z_sorted[first] for the first particle of every
    slice but the first.  Draws the reference's random.sample."""
    from random import sample
    S = n_slices
    n_part_within_cuts = n - n_cut_tail - n_cut_head
    rand_slice_i = sample(list(range(S)), n_part_within_cuts % S)
    n_part_per_slice = (n_part_within_cuts // S) * np.ones(S, dtype=np.int32)
    n_part_per_slice[rand_slice_i] += 1
    if n_part_within_cuts < S:
        raise ValueError('UniformChargeSlicer: %d particles inside the cuts '
                         'for %d slices' % (n_part_within_cuts, S))
    n_all = np.hstack((n_cut_tail, n_part_per_slice, n_cut_head))
    first_indices = np.cumsum(n_all, dtype=np.int64)[:-1]
    f = first_indices[1:-1] - n_cut_tail
    return n_part_per_slice, np.concatenate([f - 1, f])


def charge_segments(hist, ranks):
    """Tables of phk_charge_gather / _select: the coarse bin holding each
    rank becomes a segment; every rank's segment and rank inside it."""
    h = np.asarray(hist, dtype=np.int64)
    cum = np.cumsum(h)
    start = cum - h
    tb = np.searchsorted(cum, ranks, side='right')
    ub, inv = np.unique(tb, return_inverse=True)
    seg_count = h[ub]
    seg_of_bin = -np.ones(len(h), dtype=np.int32)
    seg_of_bin[ub] = np.arange(len(ub), dtype=np.int32)
    return dict(seg_of_bin=seg_of_bin, seg_count=seg_count,
                seg_off=np.concatenate([[0], np.cumsum(seg_count)[:-1]]),
                tgt_seg=inv, tgt_rank=np.asarray(ranks) - start[tb])


def charge_bins_and_edges(vals, tail, head, n_slices, code):
    """z_bins of the reference (slicing.py:661-665: midpoints between the
    last particle of a slice and the first of the next) and the lower edges
    the device bins on: the first particle of every slice, the cuts rounded
    up to the coordinate dtype at both ends."""
    S = n_slices
    lo, hi = vals[:S - 1], vals[S - 1:]
    z_bins = np.empty(S + 1)
    z_bins[1:-1] = (lo + hi) / 2
    z_bins[0], z_bins[-1] = tail, head
    edges = np.empty(S + 1, dtype=E.np_dtype(code))
    edges[0] = E.ceil_to_dtype(tail, code)
    edges[1:S] = hi
    edges[S] = E.ceil_to_dtype(head, code)
    return z_bins, edges


class UniformChargeSlicer(Slicer):
    """Slices of equal particle count over the cuts (slicing.py:618-686).

    The reference argsorts z; here the slice edges are the order statistics
    of z at the reference's ranks, found on the device without a sort
    (phk_charge_hist / _gather / _select), and the particles are then
    binned on those edges like a uniform-bin slicing.  The number of
    particles per slice follows the reference exactly, including its
    ``random.sample`` of the slices that receive one extra particle
    (Python's ``random`` module, consumed the same way).  Slice indices,
    z_bins and counts are the reference's unless two particles share a z
    value at a slice edge (the reference's assignment then depends on its
    sort's order of equal keys)."""

    def __init__(self, n_slices, n_sigma_z=None, z_cuts=None, *args,
                 **kwargs):
        if n_sigma_z and z_cuts:
            raise ValueError('Both arguments n_sigma_z and z_cuts are given '
                             'while only one is accepted!')
        if not 1 <= n_slices <= N.PHK_MAX_SLICES:
            raise ValueError('n_slices must be in [1, %d]' % N.PHK_MAX_SLICES)
        self.config = ('uniform_charge', n_slices, n_sigma_z, z_cuts)

    def times(self, z_bins, beta):
        zc = z_bins[:-1] + 0.5 * (z_bins[1:] - z_bins[:-1])
        return zc / (beta * c)

    def charge_edges(self, beam, tail, head):
        """compute_sliceset_kwargs (slicing.py:636-686) on the device:
        returns the DeviceSlicer of this slicing and its z_bins."""
        n, S = beam.macroparticlenumber, self.n_slices
        dev, code = beam._device, beam._code
        z = beam._c['z']
        stream = E.stream_handle()
        K = charge_bins_for(n)
        hist = torch.zeros(K, dtype=torch.int32, device=dev)
        below = torch.zeros(2, dtype=torch.int64, device=dev)
        N.call('phk_charge_hist', z.data_ptr(), n, code, float(tail),
               float(head), K, hist.data_ptr(), below.data_ptr(), stream)
        h = hist.cpu().numpy().astype(np.int64)
        b = below.cpu().numpy()
        n_cut_tail, n_cut_head = int(b[0]), n - int(b[1])
        per_slice, ranks = charge_ranks(n, n_cut_tail, n_cut_head, S)
        vals = np.empty(0)
        if len(ranks):
            tab = charge_segments(h, ranks)
            t = lambda a, dt: torch.from_numpy(np.ascontiguousarray(
                a, dtype=dt)).to(dev)
            d_sob = t(tab['seg_of_bin'], np.int32)
            d_off = t(tab['seg_off'], np.int64)
            d_cnt = t(tab['seg_count'], np.int32)
            d_tseg = t(tab['tgt_seg'], np.int32)
            d_trank = t(tab['tgt_rank'], np.int32)
            keys = torch.empty(max(1, int(tab['seg_count'].sum())),
                               dtype=torch.int64, device=dev)
            fill = torch.zeros(len(tab['seg_count']), dtype=torch.int32,
                               device=dev)
            status = torch.zeros(1, dtype=torch.int32, device=dev)
            out = torch.empty(len(ranks), dtype=torch.float64, device=dev)
            N.call('phk_charge_gather', z.data_ptr(), n, code, float(tail),
                   float(head), K, d_sob.data_ptr(), d_off.data_ptr(),
                   d_cnt.data_ptr(), fill.data_ptr(), keys.data_ptr(),
                   status.data_ptr(), stream)
            N.call('phk_charge_select', keys.data_ptr(), d_off.data_ptr(),
                   d_cnt.data_ptr(), d_tseg.data_ptr(), d_trank.data_ptr(),
                   len(ranks), out.data_ptr(), status.data_ptr(), stream)
            vals = out.cpu().numpy()
            if int(status.item()):
                raise N.PhkError('UniformChargeSlicer: inconsistent order '
                                 'statistics tables (device status %d)'
                                 % int(status.item()))
        z_bins, edges = charge_bins_and_edges(vals, tail, head, S, code)
        ds = E.DeviceSlicer(tail, head, S, code, dev, edges=edges)
        ds.n_part_per_slice = per_slice
        return ds, z_bins

    def slice(self, beam, *args, **kwargs):
        """Slicer.slice (slicing.py:348-381) on the GPU."""
        stats = kwargs.get('statistics', None)
        ss = make_slice_set(self, beam, with_means=bool(stats))
        if stats:
            add_statistics(ss, beam, stats)
        return ss

    def add_statistics(self, sliceset, beam, statistics):
        add_statistics(sliceset, beam, statistics)


def make_slice_set(slicer, beam, with_means=False, moments_out=None):
    """Flush the beam's pending program with a fused slicing pass and wrap
    the per-slice results in a SliceSet."""
    shards = getattr(beam, '_shard', None)
    if shards is not None and (slicer.mode == 'uniform_charge' or
                               getattr(slicer, 'z_cuts', None) is None):
        raise NotImplementedError(
            'a sharded bunch needs a uniform-bin slicer with fixed z_cuts '
            '(bunch-dependent cuts and uniform-charge slices need the whole '
            "bunch's statistics)")
    tail, head = slicer.get_long_cuts(beam)
    eng = beam._engine
    if slicer.mode == 'uniform_charge':
        # the edges follow from the z the pending program produces: run it
        # first (pending kicks do not move z and stay pending)
        if eng.ops:
            eng.flush()
        ds, z_bins = slicer.charge_edges(beam, tail, head)
    else:
        ds = slicer.device_slicer(tail, head, beam)
        z_bins = slicer.z_bins(tail, head)
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
    if shards is not None:
        from .. import shards as SH
        SH.merged_slice_moments(beam, acc, counts, mx, my, moments_out,
                                E.stream_handle())
    else:
        a = acc.struct()
        N.call('phk_slice_finalize', __import__('ctypes').byref(a),
               counts.data_ptr(), 0 if mx is None else mx.data_ptr(),
               0 if my is None else my.data_ptr(),
               0 if moments_out is None else moments_out.data_ptr(),
               E.stream_handle())
    params = Slicer.extract_beam_parameters(beam)
    params['is_sorted'] = False
    ss = SliceSet(z_bins, slicer.mode, ds, beam, counts,
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
    sh = getattr(beam, '_shard', None)
    for stat in statistics:
        if hasattr(ss, stat):
            continue
        if sh is not None and sh.world > 1:
            raise NotImplementedError(
                'slice statistic %r of a sharded bunch: only the merged '
                'mean_x and mean_y of its slicing are whole-bunch values'
                % stat)
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
