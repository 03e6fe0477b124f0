"""Particles with device-resident SoA coordinates.

Mirrors PyHEADTAIL's ``Particles`` (particles/particles.py:16-390): the same
constructor, the gamma / beta / betagamma / p0 property chain evaluated on
the host with the same NumPy formulas (so the scalars follow the
reference bit for bit, including the p0 setter round trip of
:99-104), SliceSet caching keyed by the slicer (:118-147, :210-215) and
the bunch statistics (:311-390).

The six coordinates ``x, xp, y, yp, z, dp`` are torch CUDA tensors of one
dtype: float64 (``precision='fp64'``, the plain drop-in form) or float32
(``precision='fp32'``, the precision form).  Elements of this package do
not touch them directly; they append ops to the beam's pending program
(see ``pyheadtail_gb300._engine``), which runs as one fused kernel when a
coordinate, a slice set or a statistic is needed.  Reading ``beam.x``
therefore always returns the current state.
"""
import ctypes

import numpy as np
import torch
from scipy.constants import c, e

from .. import _engine as E
from .. import _native as N
from ..general.element import Printing
from . import statistics as S

COORDS = ('x', 'xp', 'y', 'yp', 'z', 'dp')


def _as_tensor(array, dtype, device):
    if isinstance(array, torch.Tensor):
        t = array.detach().to(device=device, dtype=dtype)
        return t.clone().contiguous() if t.data_ptr() == array.data_ptr() \
            else t.contiguous()
    return torch.as_tensor(np.ascontiguousarray(array), dtype=dtype,
                           device=device).contiguous()


class Particles(Printing):
    """Beam of macroparticles; see module docstring.

    Extra keyword arguments beyond the reference's: ``precision`` ('fp64'
    or 'fp32') and ``device`` (a CUDA device, default the current one).
    """

    def __init__(self, macroparticlenumber, particlenumber_per_mp, charge,
                 mass, circumference, gamma, coords_n_momenta_dict={},
                 *args, **kwargs):
        precision = kwargs.get('precision', 'fp64')
        if precision not in ('fp64', 'fp32'):
            raise ValueError("precision must be 'fp64' or 'fp32'")
        if not torch.cuda.is_available():
            raise N.PhkError('pyheadtail_gb300.Particles needs a CUDA device '
                             '(sm_103a); there is no CPU path')
        N.load()
        self.precision = precision
        self._code = N.PHK_F64 if precision == 'fp64' else N.PHK_F32
        self._dtype = E.torch_dtype(self._code)
        self._device = torch.device(kwargs.get('device', 'cuda'))
        self._c = {}
        self._engine = E.Engine(self)
        self._exposed = 0          # bumped when a coordinate is handed out
        self._rebinds = 0          # bumped when a coordinate array is replaced
        self._stats_ws = None
        self._stats_cache = None
        self._stats_mask = 0
        self._stats_order = 1
        self.macroparticlenumber = int(macroparticlenumber)
        self.particlenumber_per_mp = particlenumber_per_mp
        self.charge = charge
        self.mass = mass
        self.circumference = circumference
        self.gamma = gamma
        self._slice_sets = {}
        self.coords_n_momenta = set()
        self.id = torch.arange(1, self.macroparticlenumber + 1,
                               dtype=torch.int32, device=self._device)
        self.update(coords_n_momenta_dict)

    # -------------------------------------------------- scalar properties
    @property
    def intensity(self):
        return self.particlenumber_per_mp * self.macroparticlenumber

    @intensity.setter
    def intensity(self, value):
        self.particlenumber_per_mp = value / float(self.macroparticlenumber)

    @property
    def charge_per_mp(self):
        return self.particlenumber_per_mp * self.charge

    @charge_per_mp.setter
    def charge_per_mp(self, value):
        self.particlenumber_per_mp = value / self.charge

    @property
    def gamma(self):
        return self._gamma

    @gamma.setter
    def gamma(self, value):
        self._gamma = value
        self._beta = np.sqrt(1 - self.gamma**-2)
        self._betagamma = np.sqrt(self.gamma**2 - 1)
        self._p0 = self.betagamma * self.mass * c

    @property
    def beta(self):
        return self._beta

    @beta.setter
    def beta(self, value):
        self.gamma = 1. / np.sqrt(1 - value**2)

    @property
    def betagamma(self):
        return self._betagamma

    @betagamma.setter
    def betagamma(self, value):
        self.gamma = np.sqrt(value**2 + 1)

    @property
    def p0(self):
        return self._p0

    @p0.setter
    def p0(self, value):
        self.gamma = np.sqrt(1 + (value / (self.mass * c))**2)

    # -------------------------------------------------- coordinates
    def _get(self, name):
        if name not in self._c:
            raise AttributeError(name)
        self._engine.sync_for(name)
        self._exposed += 1
        return self._c[name]

    def _set(self, name, value):
        if name in self._c and value is self._c[name]:
            return
        self._engine.flush()
        self._engine.z_version += 1
        self._exposed += 1
        self._rebinds += 1
        t = _as_tensor(value, self._dtype, self._device)
        if t.shape != (self.macroparticlenumber,):
            raise ValueError('lengths of given phase space coordinate arrays '
                             'do not coincide with self.macroparticlenumber.')
        self._c[name] = t

    x = property(lambda s: s._get('x'), lambda s, v: s._set('x', v))
    xp = property(lambda s: s._get('xp'), lambda s, v: s._set('xp', v))
    y = property(lambda s: s._get('y'), lambda s, v: s._set('y', v))
    yp = property(lambda s: s._get('yp'), lambda s, v: s._set('yp', v))
    z = property(lambda s: s._get('z'), lambda s, v: s._set('z', v))
    dp = property(lambda s: s._get('dp'), lambda s, v: s._set('dp', v))

    @property
    def z_beamframe(self):
        return self.z * self.gamma

    @z_beamframe.setter
    def z_beamframe(self, value):
        self.z = value / self.gamma

    def get_coords_n_momenta_dict(self):
        return {k: getattr(self, k) for k in self.coords_n_momenta}

    def update(self, coords_n_momenta_dict):
        """particles/particles.py:217-229 (copies the arrays to the device)."""
        if any(len(v) != self.macroparticlenumber
               for v in coords_n_momenta_dict.values()):
            raise ValueError('lengths of given phase space coordinate arrays '
                             'do not coincide with self.macroparticlenumber.')
        for k, v in coords_n_momenta_dict.items():
            if k in COORDS:
                self._set(k, v)
            else:
                setattr(self, k, _as_tensor(v, self._dtype, self._device))
        self.coords_n_momenta.update(coords_n_momenta_dict.keys())

    def add(self, coords_n_momenta_dict):
        if any(s in self.coords_n_momenta for s in coords_n_momenta_dict):
            raise ValueError('One or more of the specified coordinates or '
                             'momenta already exist and cannot be added. Use '
                             'self.update(...) for this purpose.')
        self.update(coords_n_momenta_dict)

    def coords_numpy(self):
        """float64 NumPy copies of the six coordinates (synchronises)."""
        return {k: getattr(self, k).double().cpu().numpy() for k in COORDS
                if k in self._c}

    def sort_for(self, attr):
        self.reorder(torch.argsort(getattr(self, attr)))

    def reorder(self, permutation, except_for_attrs=[]):
        self._engine.flush()
        self._exposed += 1
        self._rebinds += 1
        for attr in ['id'] + list(self.coords_n_momenta):
            if attr in except_for_attrs:
                continue
            if attr in COORDS:
                self._c[attr] = self._c[attr][permutation].contiguous()
            else:
                setattr(self, attr, getattr(self, attr)[permutation])
        self.clean_slices()

    # -------------------------------------------------- slicing
    def get_slices(self, slicer, *args, **kwargs):
        """particles/particles.py:118-147."""
        if slicer not in self._slice_sets or kwargs.get('statistics'):
            self._slice_sets[slicer] = slicer.slice(self, *args, **kwargs)
        return self._slice_sets[slicer]

    def clean_slices(self):
        self._slice_sets = {}

    def _empty_like(self, macroparticlenumber):
        """A beam with this one's scalars, precision and device and no
        coordinates yet."""
        return Particles(macroparticlenumber, self.particlenumber_per_mp,
                         self.charge, self.mass, self.circumference,
                         self.gamma, coords_n_momenta_dict={},
                         precision=self.precision, device=self._device)

    def extract_slices(self, slicer, include_non_sliced='if_any', *args,
                       **kwargs):
        """One Particles per slice, plus one of the particles outside the
        cuts (particles/particles.py:150-207), each with ``slice_info``."""
        if include_non_sliced not in ['if_any', 'always', 'never']:
            raise ValueError("include_non_sliced=%s is not valid!\n"
                             % include_non_sliced +
                             "Possible values are {'always', 'never', "
                             "'if_any'}")
        slices = self.get_slices(slicer, *args, **kwargs)
        _ = slices.slice_index_of_particle  # taken while z is the sliced one
        coords = self.get_coords_n_momenta_dict()
        out = []
        for i_sl in range(slices.n_slices):
            ix = slices.particle_indices_of_slice(i_sl).long()
            so = self._empty_like(len(ix))
            so.update({k: v[ix] for k, v in coords.items()})
            so.id[:] = self.id[ix]
            so.slice_info = {'z_bin_center': slices.z_centers[i_sl],
                             'z_bin_right': slices.z_bins[i_sl + 1],
                             'z_bin_left': slices.z_bins[i_sl]}
            out.append(so)
        if include_non_sliced != 'never':
            ix = slices.particles_outside_cuts.long()
            if len(ix) > 0 or include_non_sliced == 'always':
                so = self._empty_like(len(ix))
                so.update({k: v[ix] for k, v in coords.items()})
                so.id[:] = self.id[ix]
                so.slice_info = 'unsliced'
                out.append(so)
        return out

    def __add__(self, other):
        """Merges two beams: coordinates and ids concatenated, the scalars
        of the left one (particles/particles.py:264-288)."""
        a = self.get_coords_n_momenta_dict()
        b = other.get_coords_n_momenta_dict()
        result = self._empty_like(self.macroparticlenumber +
                                  other.macroparticlenumber)
        result.update({k: torch.cat((a[k], b[k].to(device=a[k].device,
                                                     dtype=a[k].dtype)))
                       for k in a})
        result.id = torch.cat((self.id, other.id.to(self.id.device)))
        return result

    def __radd__(self, other):
        """``0 + beam`` is a copy of the beam (so that sum() works),
        anything else merges (particles/particles.py:290-305)."""
        if other == 0:
            result = self._empty_like(self.macroparticlenumber)
            result.update({k: v.clone() for k, v in
                           self.get_coords_n_momenta_dict().items()})
            result.id = self.id.clone()
            return result
        return self.__add__(other)

    # -------------------------------------------------- statistics
    # Every statistic is derived from one phk_bunch_stats record of the
    # current state: one read-only pass over the coordinates, with the
    # pending wake kicks applied in registers (no kick pass is forced), and
    # one 272-byte read back.  A record stays valid until the state
    # changes (an element enqueues an op or a kick, a coordinate is set or
    # handed out); the coordinates and the order asked for so far are
    # remembered, so a loop asking the same statistics every turn costs one
    # pass per turn.
    def _stats_workspace(self):
        if self._stats_ws is None:
            grid = N.call('phk_bunch_stats_grid', self.macroparticlenumber,
                          self._code)
            dev = self._device
            part = torch.empty(grid * S.RECORD_LEN, dtype=torch.float64,
                               device=dev)
            ticket = torch.zeros(1, dtype=torch.int32, device=dev)
            rec = torch.empty(S.RECORD_LEN, dtype=torch.float64, device=dev)
            self._stats_ws = (grid, part, ticket, rec)
        return self._stats_ws

    def stats_struct(self, records, capacity=1, cursor=None, order=2,
                     mask=0x3f, means=None):
        """phk_stats for a statistics pass of this bunch into ``records``
        (a float64 CUDA tensor of capacity * 34 entries); ``means`` (a
        float64 CUDA tensor of 9 entries) receives the device means."""
        grid, part, ticket, _ = self._stats_workspace()
        st = N.Stats()
        st.order = order
        st.capacity = capacity
        st.records = records.data_ptr()
        st.cursor = 0 if cursor is None else cursor.data_ptr()
        st.partials = part.data_ptr()
        st.ticket = ticket.data_ptr()
        st.means = 0 if means is None else means.data_ptr()
        st.grid = grid
        st.mask = mask
        return st

    def launch_stats(self, records, capacity=1, cursor=None, order=2,
                     mask=0x3f, means=None):
        """Queue one statistics pass of the current state (no sync)."""
        eng = self._engine
        if eng.ops:
            eng.flush()
        st = self.stats_struct(records, capacity, cursor, order, mask, means)
        coords = eng.coords_struct()
        ks = eng.kick.struct() if eng.kick is not None else None
        N.call('phk_bunch_stats', ctypes.byref(coords),
               ctypes.byref(ks) if ks is not None else None,
               ctypes.byref(st), E.stream_handle())
        eng.launches += 1

    def _state_key(self):
        return (self._exposed, self._engine.version)

    def _stats_record(self, coords, order):
        key = self._state_key()
        cached = self._stats_cache
        if cached is not None and cached[0] == key and \
                cached[1].covers(coords, order):
            return cached[1]
        self._stats_mask |= S.mask_of(coords)
        self._stats_order = max(self._stats_order, order)
        rec = self._stats_workspace()[3]
        self.launch_stats(rec, order=self._stats_order, mask=self._stats_mask)
        r = S.StatsRecord(rec.cpu().numpy(), self._stats_mask,
                          self._stats_order)
        self._stats_cache = (key, r)
        return r

    def _statistic(self, name):
        coords, order = S.NEEDS[name]
        r = self._stats_record(coords, order)
        return r.statistic(name, self.betagamma, self.p0, e)

    def mean_x(self, **kwargs):
        return self._statistic('mean_x')

    def mean_xp(self, **kwargs):
        return self._statistic('mean_xp')

    def mean_y(self, **kwargs):
        return self._statistic('mean_y')

    def mean_yp(self, **kwargs):
        return self._statistic('mean_yp')

    def mean_z(self, **kwargs):
        return self._statistic('mean_z')

    def mean_dp(self, **kwargs):
        return self._statistic('mean_dp')

    def sigma_x(self, **kwargs):
        return self._statistic('sigma_x')

    def sigma_y(self, **kwargs):
        return self._statistic('sigma_y')

    def sigma_z(self, **kwargs):
        return self._statistic('sigma_z')

    def sigma_xp(self, **kwargs):
        return self._statistic('sigma_xp')

    def sigma_yp(self, **kwargs):
        return self._statistic('sigma_yp')

    def sigma_dp(self, **kwargs):
        return self._statistic('sigma_dp')

    def effective_normalized_emittance_x(self, **kwargs):
        return self._statistic('effective_normalized_emittance_x')

    def effective_normalized_emittance_y(self, **kwargs):
        return self._statistic('effective_normalized_emittance_y')

    def effective_normalized_emittance_z(self, **kwargs):
        return self._statistic('effective_normalized_emittance_z')

    def epsn_x(self, **kwargs):
        return self._statistic('epsn_x')

    def epsn_y(self, **kwargs):
        return self._statistic('epsn_y')

    def epsn_z(self, **kwargs):
        # always the effective emittance (particles.py:363-365)
        return self._statistic('epsn_z')

    def dispersion_x(self):
        return self._statistic('dispersion_x')

    def dispersion_y(self):
        return self._statistic('dispersion_y')

    def alpha_Twiss_x(self):
        return self._statistic('alpha_Twiss_x')

    def alpha_Twiss_y(self):
        return self._statistic('alpha_Twiss_y')

    def beta_Twiss_x(self):
        return self._statistic('beta_Twiss_x')

    def beta_Twiss_y(self):
        return self._statistic('beta_Twiss_y')

    def gamma_Twiss_x(self):
        return self._statistic('gamma_Twiss_x')

    def gamma_Twiss_y(self):
        return self._statistic('gamma_Twiss_y')
