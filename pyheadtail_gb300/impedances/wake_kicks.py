"""Wake kicks for the GPU turn loop.

Mirrors PyHEADTAIL's impedances/wake_kicks.py: the ``WakeKick`` base
(:19-139: convolution path choice :41-53, ``_wake_factor`` :66-73, the two
convolutions :75-116, the multi-turn accumulation :118-139) and the
constant (:144-202), dipolar (:207-279) and quadrupolar (:284-361) kicks.

The wake function is evaluated on the host with the reference's NumPy
formula at exactly the time differences the reference uses, once per
(target times, source times, age, beta) -- for fixed cuts and constant
energy that is once per stored turn for the whole run -- and kept on the
device.  The convolution over all stored turns runs in ``phk_wake``; the
resulting per-slice kick is left pending on the beam and applied to the
particles at the start of the next fused pass.
"""
from abc import ABCMeta

import numpy as np
import torch
from scipy.constants import c

from .. import _native as N
from ..general.element import Printing

# source moment of each kick type: 0 count, 1 count*mean_x, 2 count*mean_y
_SOURCE = {'count': 0, 'x': 1, 'y': 2}


class WakeKick(Printing, metaclass=ABCMeta):
    """Base: path choice, wake factor and table management."""

    target = None   # 'xp' | 'yp' | 'dp'
    moment = None   # 'count' | 'x' | 'y'
    quad = None     # None | 'x' | 'y' (quadrupolar: kick * coordinate)

    def __init__(self, wake_function, slicer, n_turns_wake, *args, **kwargs):
        self.wake_function = wake_function
        if (slicer.mode == 'uniform_bin' and
                (n_turns_wake == 1 or slicer.z_cuts)):
            self._dense = False
        else:
            self._dense = True
            if n_turns_wake > 1:
                self.warns('You use multiturn wakes. The stored SliceSet '
                           'instances from previous turns are converted from '
                           'z to dt according to the current turn\'s gamma. '
                           'If you accelerate this is only an approximation '
                           'which becomes invalid when gamma changes much '
                           'over n_turns_wake.')
        self.n_turns_wake = n_turns_wake
        self._table = None
        self._keys = []

    @staticmethod
    def _wake_factor(bunch):
        """wake_kicks.py:66-73."""
        return (-(bunch.charge)**2 / (bunch.mass * bunch.gamma *
                (bunch.beta * c)**2) * bunch.particlenumber_per_mp)

    # -- host-side wake samples, exactly the reference's time differences
    def _samples(self, target_times, source_times, source_beta):
        if self._dense:
            dt = [target_times] - np.transpose([source_times])
        else:
            dt = np.concatenate((target_times - source_times[-1],
                                 (target_times - source_times[0])[1:]))
        return self.wake_function(dt, beta=source_beta)

    def _sync_tables(self, times, ages, betas, n_slices, device):
        """Make table[a] = wake samples of stored turn a for every lag in
        use; upload only the lags whose inputs changed."""
        n_lags = min(len(ages), self.n_turns_wake)
        width = n_slices * n_slices if self._dense else 2 * n_slices - 1
        if (self._table is None or self._table.shape[1] != width or
                self._table.device != device):
            self._table = torch.zeros(self.n_turns_wake, width,
                                      dtype=torch.float64, device=device)
            self._keys = [None] * self.n_turns_wake
        for a in range(n_lags):
            key = (times[0], times[a], float(ages[a]), float(betas[a]))
            old = self._keys[a]
            if (old is not None and old[0] is key[0] and old[1] is key[1]
                    and old[2] == key[2] and old[3] == key[3]):
                continue
            w = self._samples(times[0], times[a] + ages[a], betas[a])
            self._table[a].copy_(torch.from_numpy(
                np.ascontiguousarray(w, dtype=np.float64).ravel()))
            self._keys[a] = key
        return n_lags

    def _fill(self, st, bunch, slice_sets, ages, out):
        """Fill the phk_wake_kick block of this kick for the current turn."""
        times = [s._times for s in slice_sets]
        betas = [s.beta for s in slice_sets]
        n_slices = slice_sets[0].n_slices
        st.n_lags = self._sync_tables(times, ages, betas, n_slices,
                                      out.device)
        st.source = _SOURCE[self.moment]
        st.dense = int(self._dense)
        st.factor = float(self._wake_factor(bunch))
        st.table = self._table.data_ptr()
        st.out = out.data_ptr()

    def pending_entry(self, out):
        q = None if self.quad is None else N.COORD_INDEX[self.quad]
        return (N.COORD_INDEX[self.target], q, out)

    def apply(self, bunch, slice_set_list, slice_set_age_list):
        """Standalone use (outside a WakeField): convolve and kick now."""
        from .wakes import _run_kicks
        _run_kicks([self], bunch, slice_set_list, slice_set_age_list)


class ConstantWakeKickX(WakeKick):
    target, moment = 'xp', 'count'


class ConstantWakeKickY(WakeKick):
    target, moment = 'yp', 'count'


class ConstantWakeKickZ(WakeKick):
    target, moment = 'dp', 'count'


class DipoleWakeKickX(WakeKick):
    target, moment = 'xp', 'x'


class DipoleWakeKickXY(WakeKick):
    target, moment = 'xp', 'y'


class DipoleWakeKickY(WakeKick):
    target, moment = 'yp', 'y'


class DipoleWakeKickYX(WakeKick):
    target, moment = 'yp', 'x'


class QuadrupoleWakeKickX(WakeKick):
    target, moment, quad = 'xp', 'count', 'x'


class QuadrupoleWakeKickXY(WakeKick):
    target, moment, quad = 'xp', 'count', 'y'


class QuadrupoleWakeKickY(WakeKick):
    target, moment, quad = 'yp', 'count', 'y'


class QuadrupoleWakeKickYX(WakeKick):
    target, moment, quad = 'yp', 'count', 'x'
