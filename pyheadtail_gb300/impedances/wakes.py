"""Wake fields and wake sources for the GPU turn loop.

Mirrors PyHEADTAIL's impedances/wakes.py: ``WakeField`` (:77-145),
``WakeSource`` (:150-163), ``Resonator`` (:379-493) with its circular and
parallel-plates variants (:496-548) and ``ResistiveWall`` (:551-624) with
its variants (:627-678), same constructors and the same
``get_wake_kicks`` order.  The wake functions are the reference formulas
(NumPy, evaluated on the host into device tables).

``WakeField.track(bunch)``, per turn:
  1. ages of the stored slice sets += C / (beta c)          (wakes.py:135-137)
  2. one fused pass: pending kicks + pending program + slicing; the fixed-
     order merge writes counts, mean_x, mean_y and the moment ring slot
  3. ``phk_wake``: every kick's multi-turn convolution on the device (FP32
     form: ``phk_wake_tc_run``, a BF16x3 Toeplitz GEMM on the tensor cores)
  4. the kicks are left pending on the beam (applied by the next pass).
``WakeTable`` (:167-376) samples tabulated wakes with the reference's
interpolation on the host; the device work is the same.
"""
import ctypes
from abc import ABCMeta, abstractmethod
from collections import deque

import numpy as np
import torch
from scipy.constants import c

from .. import _engine as E
from .. import _native as N
from ..general.element import Element, Printing
from ..particles.slicing import make_slice_set
from .wake_kicks import (ConstantWakeKickZ, DipoleWakeKickX, DipoleWakeKickY,
                         QuadrupoleWakeKickX, QuadrupoleWakeKickY)

sin = np.sin
cos = np.cos


class _RingState(object):
    """Device ring of per-slice moments + kick outputs of one WakeField."""

    def __init__(self, n_ring, n_slices, n_kicks, code, device):
        self.n_ring, self.n_slices = n_ring, n_slices
        self.code, self.device = code, device
        self.moments = torch.zeros(n_ring, 3, n_slices, dtype=torch.float64,
                                   device=device)
        self.kick_out = torch.zeros(max(n_kicks, 1), n_slices,
                                    dtype=E.torch_dtype(code), device=device)
        self.head = -1
        self.tensor = None

    def matches(self, n_slices, code, device):
        return (self.n_slices == n_slices and self.code == code and
                self.device == device)


class _TensorWake(object):
    """Tensor-core convolution (phk_wake_tc_*) of the kicks of one WakeField
    in the FP32 form.  Kicks whose sampled tables are equal share a table
    group; the bfloat16 high / low parts of the tables are rewritten
    whenever a table changes (for fixed cuts and energy: during the first
    n_turns_wake turns); the GEMM builds its Toeplitz tiles from them."""

    def __init__(self, device):
        self.device = device
        self._sig = None
        self.w = None

    @staticmethod
    def signature(kicks):
        return tuple((id(k._table), tuple(
            None if key is None else (id(key[0]), id(key[1]), key[2], key[3])
            for key in k._keys)) for k in kicks)

    def _regroup(self, kicks, n_slices):
        reps, group_of = [], []
        for k in kicks:
            for g, r in enumerate(reps):
                if r._table.shape == k._table.shape and \
                        torch.equal(r._table, k._table):
                    group_of.append(g)
                    break
            else:
                group_of.append(len(reps))
                reps.append(k)
        w = N.WakeTC()
        w.n_slices = n_slices
        w.n_kicks = len(kicks)
        w.n_groups = len(reps)
        for g, r in enumerate(reps):
            w.group_lags[g] = r.n_turns_wake
            w.tables[g] = r._table.data_ptr()
        for i, g in enumerate(group_of):
            w.group_of[i] = g
        a_el, p_el = ctypes.c_int64(), ctypes.c_int64()
        N.call('phk_wake_tc_plan', ctypes.byref(w), ctypes.byref(a_el),
               ctypes.byref(p_el))
        if self.w is None or self.a_hi.numel() != a_el.value:
            self.a_hi = torch.empty(a_el.value, dtype=torch.int16,
                                    device=self.device)
            self.a_lo = torch.empty(a_el.value, dtype=torch.int16,
                                    device=self.device)
        if self.w is None or self.partials.numel() != p_el.value:
            self.partials = torch.empty(p_el.value, dtype=torch.float32,
                                        device=self.device)
        w.a_hi = self.a_hi.data_ptr()
        w.a_lo = self.a_lo.data_ptr()
        w.partials = self.partials.data_ptr()
        self.w = w
        self.reps = reps

    def run(self, kicks, ws):
        sig = self.signature(kicks)
        if sig != self._sig:
            self._regroup(kicks, ws.n_slices)
            N.call('phk_wake_tc_expand', ctypes.byref(self.w),
                   E.stream_handle())
            self._sig = sig
        w = self.w
        w.ring_len, w.head = ws.ring_len, ws.head
        w.out_dtype = ws.out_dtype
        w.moments = ws.moments
        for k in range(len(kicks)):
            st = ws.kick[k]
            w.source[k] = st.source
            w.n_lags[k] = st.n_lags
            w.factor[k] = st.factor
            w.out[k] = st.out
        N.call('phk_wake_tc_run', ctypes.byref(w), E.stream_handle())


def _tensor_path(kicks, bunch):
    """FP32 form, a multi-turn wake and every kick on the convolution path:
    the wake runs as a tensor-core GEMM.  A single-turn convolution (K = S)
    is too small to amortise the GEMM's staging and stays on phk_wake."""
    return (bunch._code == N.PHK_F32 and 0 < len(kicks) <= N.PHK_MAX_KICKS
            and not any(k._dense for k in kicks)
            and max(k.n_turns_wake for k in kicks) > 1)


def _run_kicks(kicks, bunch, slice_sets, ages, state=None):
    """Convolve every kick (phk_wake) and leave the kicks pending."""
    ss = slice_sets[0]
    if state is None:
        state = getattr(ss, '_ring', None)
    if state is None:
        raise RuntimeError('slice sets made outside a WakeField carry no '
                           'moment ring; track through a WakeField')
    ws = N.WakeSet()
    ws.n_slices = ss.n_slices
    ws.ring_len = state.n_ring
    ws.head = state.head
    ws.n_kicks = len(kicks)
    ws.out_dtype = bunch._code
    ws.moments = state.moments.data_ptr()
    entries = []
    for k, kick in enumerate(kicks):
        out = state.kick_out[k]
        kick._fill(ws.kick[k], bunch, slice_sets, ages, out)
        entries.append(kick.pending_entry(out))
    if _tensor_path(kicks, bunch):
        if getattr(state, 'tensor', None) is None:
            state.tensor = _TensorWake(state.moments.device)
        state.tensor.run(kicks, ws)
    else:
        N.call('phk_wake', ctypes.byref(ws), E.stream_handle())
    bunch._engine.set_kick(E.PendingKick(ss._dslicer, entries))


class WakeField(Element):
    """Collection of wake kicks sharing one slicer and a multi-turn slice
    set history (wakes.py:77-145)."""

    def __init__(self, slicer, *wake_sources):
        self.slicer = slicer
        self.wake_kicks = []
        for source in wake_sources:
            self.wake_kicks.extend(source.get_wake_kicks(self.slicer))
        if len(self.wake_kicks) > N.PHK_MAX_KICKS:
            raise ValueError('at most %d wake kicks per WakeField'
                             % N.PHK_MAX_KICKS)
        n_turns_wake_max = max([source.n_turns_wake
                                for source in wake_sources])
        self.slice_set_deque = deque([], maxlen=n_turns_wake_max)
        self.slice_set_age_deque = deque([], maxlen=n_turns_wake_max)
        self._state = None

    def _ring(self, bunch):
        S = self.slicer.n_slices
        st = self._state
        if st is None or not st.matches(S, bunch._code, bunch._device):
            st = _RingState(self.slice_set_deque.maxlen, S,
                            len(self.wake_kicks), bunch._code, bunch._device)
            self._state = st
            self.slice_set_deque.clear()
            self.slice_set_age_deque.clear()
        return st

    def track(self, bunch):
        for i in range(len(self.slice_set_age_deque)):
            self.slice_set_age_deque[i] += (
                bunch.circumference / (bunch.beta * c))
        st = self._ring(bunch)
        st.head = (st.head + 1) % st.n_ring
        slice_set = make_slice_set(self.slicer, bunch, with_means=True,
                                   moments_out=st.moments[st.head])
        slice_set._times = self.slicer.times(slice_set.z_bins, slice_set.beta)
        slice_set._ring = st
        bunch._slice_sets[self.slicer] = slice_set
        self.slice_set_deque.appendleft(slice_set)
        self.slice_set_age_deque.appendleft(0.)
        if self.wake_kicks:
            _run_kicks(self.wake_kicks, bunch, self.slice_set_deque,
                       self.slice_set_age_deque, st)


class WakeSource(Printing, metaclass=ABCMeta):

    @abstractmethod
    def get_wake_kicks(self, slicer_mode):
        pass


class Resonator(WakeSource):
    """Resonator wake (Chao eq. 2.82, HEADTAIL conventions),
    wakes.py:379-493."""

    def __init__(self, R_shunt, frequency, Q, Yokoya_X1, Yokoya_Y1,
                 Yokoya_X2, Yokoya_Y2, switch_Z, n_turns_wake=1, *args,
                 **kwargs):
        self.R_shunt = R_shunt
        self.frequency = frequency
        self.Q = Q
        self.Yokoya_X1 = Yokoya_X1
        self.Yokoya_X2 = Yokoya_X2
        self.Yokoya_Y1 = Yokoya_Y1
        self.Yokoya_Y2 = Yokoya_Y2
        self.switch_Z = switch_Z
        self.n_turns_wake = n_turns_wake

    def get_wake_kicks(self, slicer):
        kicks = []
        if self.Yokoya_X1:
            kicks.append(DipoleWakeKickX(
                self.function_transverse(self.Yokoya_X1), slicer,
                self.n_turns_wake))
        if self.Yokoya_X2:
            kicks.append(QuadrupoleWakeKickX(
                self.function_transverse(self.Yokoya_X2), slicer,
                self.n_turns_wake))
        if self.Yokoya_Y1:
            kicks.append(DipoleWakeKickY(
                self.function_transverse(self.Yokoya_Y1), slicer,
                self.n_turns_wake))
        if self.Yokoya_Y2:
            kicks.append(QuadrupoleWakeKickY(
                self.function_transverse(self.Yokoya_Y2), slicer,
                self.n_turns_wake))
        if self.switch_Z:
            kicks.append(ConstantWakeKickZ(
                self.function_longitudinal(), slicer, self.n_turns_wake))
        return kicks

    def function_transverse(self, Yokoya_factor):
        """wakes.py:450-470."""
        omega = 2 * np.pi * self.frequency
        alpha = omega / (2 * self.Q)
        omegabar = np.sqrt(np.abs(omega**2 - alpha**2))

        def wake(dt, *args, **kwargs):
            dt = dt.clip(max=0)
            if self.Q > 0.5:
                y = (Yokoya_factor * self.R_shunt * omega**2 /
                     (self.Q * omegabar) * np.exp(alpha * dt) *
                     sin(omegabar * dt))
            elif self.Q == 0.5:
                y = (Yokoya_factor * self.R_shunt * omega**2 / self.Q *
                     np.exp(alpha * dt) * dt)
            else:
                y = (Yokoya_factor * self.R_shunt * omega**2 /
                     (self.Q * omegabar) * np.exp(alpha * dt) *
                     np.sinh(omegabar * dt))
            return y
        return wake

    def function_longitudinal(self):
        """wakes.py:472-493."""
        omega = 2 * np.pi * self.frequency
        alpha = omega / (2 * self.Q)
        omegabar = np.sqrt(np.abs(omega**2 - alpha**2))

        def wake(dt, *args, **kwargs):
            if self.Q > 0.5:
                y = (-(np.sign(dt) - 1) * self.R_shunt * alpha *
                     np.exp(alpha * dt) * (cos(omegabar * dt) +
                     alpha / omegabar * sin(omegabar * dt)))
            elif self.Q == 0.5:
                y = (-(np.sign(dt) - 1) * self.R_shunt * alpha *
                     np.exp(alpha * dt) * (1. + alpha * dt))
            elif self.Q < 0.5:
                y = (-(np.sign(dt) - 1) * self.R_shunt * alpha *
                     np.exp(alpha * dt) * (np.cosh(omegabar * dt) +
                     alpha / omegabar * np.sinh(omegabar * dt)))
            return y
        return wake


class CircularResonator(Resonator):
    def __init__(self, R_shunt, frequency, Q, n_turns_wake=1, *args,
                 **kwargs):
        super(CircularResonator, self).__init__(
            R_shunt, frequency, Q, 1., 1., 0., 0., False, n_turns_wake,
            *args, **kwargs)


class ParallelHorizontalPlatesResonator(Resonator):
    def __init__(self, R_shunt, frequency, Q, n_turns_wake=1, *args,
                 **kwargs):
        super(ParallelHorizontalPlatesResonator, self).__init__(
            R_shunt, frequency, Q, np.pi**2 / 24., np.pi**2 / 12.,
            -np.pi**2 / 24., np.pi**2 / 24., False, n_turns_wake, *args,
            **kwargs)


class ParallelPlatesResonator(ParallelHorizontalPlatesResonator):
    pass


class ParallelVerticalPlatesResonator(Resonator):
    def __init__(self, R_shunt, frequency, Q, n_turns_wake=1, *args,
                 **kwargs):
        super(ParallelVerticalPlatesResonator, self).__init__(
            R_shunt, frequency, Q, np.pi**2 / 12., np.pi**2 / 24.,
            np.pi**2 / 24., -np.pi**2 / 24., False, n_turns_wake, *args,
            **kwargs)


class ResistiveWall(WakeSource):
    """Resistive-wall wake (wakes.py:551-624)."""

    def __init__(self, pipe_radius, resistive_wall_length, conductivity,
                 dt_min, Yokoya_X1, Yokoya_Y1, Yokoya_X2, Yokoya_Y2,
                 n_turns_wake=1, *args, **kwargs):
        self.pipe_radius = np.array([pipe_radius]).flatten()
        self.resistive_wall_length = resistive_wall_length
        self.conductivity = conductivity
        self.dt_min = dt_min
        self.Yokoya_X1 = Yokoya_X1
        self.Yokoya_Y1 = Yokoya_Y1
        self.Yokoya_X2 = Yokoya_X2
        self.Yokoya_Y2 = Yokoya_Y2
        self.n_turns_wake = n_turns_wake

    def get_wake_kicks(self, slicer):
        kicks = []
        if self.Yokoya_X1:
            kicks.append(DipoleWakeKickX(
                self.function_transverse(self.Yokoya_X1), slicer,
                self.n_turns_wake))
        if self.Yokoya_X2:
            kicks.append(QuadrupoleWakeKickX(
                self.function_transverse(self.Yokoya_X2), slicer,
                self.n_turns_wake))
        if self.Yokoya_Y1:
            kicks.append(DipoleWakeKickY(
                self.function_transverse(self.Yokoya_Y1), slicer,
                self.n_turns_wake))
        if self.Yokoya_Y2:
            kicks.append(QuadrupoleWakeKickY(
                self.function_transverse(self.Yokoya_Y2), slicer,
                self.n_turns_wake))
        return kicks

    def function_transverse(self, Yokoya_factor):
        """wakes.py:611-624."""
        mu_r = 1
        Z_0 = 119.9169832 * np.pi

        def wake(dt, *args, **kwargs):
            y = (Yokoya_factor * (np.sign(dt + np.abs(self.dt_min)) - 1) / 2. *
                 np.sqrt(kwargs['beta']) * self.resistive_wall_length /
                 np.pi / self.pipe_radius**3 * np.sqrt(
                     -mu_r / np.pi / self.conductivity /
                     dt.clip(max=-abs(self.dt_min)))) * np.sqrt(Z_0 * c)
            return y
        return wake


class CircularResistiveWall(ResistiveWall):
    def __init__(self, pipe_radius, resistive_wall_length, conductivity,
                 dt_min, n_turns_wake=1, *args, **kwargs):
        super(CircularResistiveWall, self).__init__(
            pipe_radius, resistive_wall_length, conductivity, dt_min, 1., 1.,
            0., 0., n_turns_wake, *args, **kwargs)


class ParallelHorizontalPlatesResistiveWall(ResistiveWall):
    def __init__(self, pipe_radius, resistive_wall_length, conductivity,
                 dt_min, n_turns_wake=1, *args, **kwargs):
        super(ParallelHorizontalPlatesResistiveWall, self).__init__(
            pipe_radius, resistive_wall_length, conductivity, dt_min,
            np.pi**2 / 24., np.pi**2 / 12., -np.pi**2 / 24., np.pi**2 / 24.,
            n_turns_wake, *args, **kwargs)


class ParallelPlatesResistiveWall(ParallelHorizontalPlatesResistiveWall):
    pass


class ParallelVerticalPlatesResistiveWall(ResistiveWall):
    """Note: the reference derives this class from Resonator
    (wakes.py:664-678), which misplaces its arguments; here it is the
    resistive wall its name describes."""

    def __init__(self, pipe_radius, resistive_wall_length, conductivity,
                 dt_min, n_turns_wake=1, *args, **kwargs):
        super(ParallelVerticalPlatesResistiveWall, self).__init__(
            pipe_radius, resistive_wall_length, conductivity, dt_min,
            np.pi**2 / 12., np.pi**2 / 24., np.pi**2 / 24., -np.pi**2 / 24.,
            n_turns_wake, *args, **kwargs)


class WakeTable(WakeSource):
    """Wakes from a table (wakes.py:167-376): the same file format and
    column names, the same get_wake_kicks order, and the reference's
    linear interpolation (scipy interp1d of the table converted to SI
    units and HEADTAIL signs), evaluated on the host into the device
    tables of the convolution.

    Columns (``wake_file_columns``, in file order): 'time' [ns] and any of
    'constant_x', 'constant_y', 'dipole_x', 'dipole_y', 'dipole_xy',
    'dipole_yx', 'quadrupole_x', 'quadrupole_y', 'quadrupole_xy',
    'quadrupole_yx' [V/pC/mm] and 'longitudinal' [V/pC].  A table whose
    first time is 0 (with transverse values 0 there) is an
    ultrarelativistic wake, clipped to dt <= 0; a table starting at
    negative times is a low-beta wake.  Transverse samples outside the
    table raise ValueError (interp1d), longitudinal ones are 0.
    One difference: the reference appends a 'quadrupole_xy' kick to a
    list that does not exist (wakes.py:274-277) and so raises; here the
    kick is created like the others."""

    def __init__(self, wake_file, wake_file_columns, n_turns_wake=1, *args,
                 **kwargs):
        self.wake_table = {}
        wake_data = np.loadtxt(wake_file)
        if len(wake_file_columns) != wake_data.shape[1]:
            raise ValueError('Length of wake_file_columns list does not '
                             'correspond to the number of columns in the '
                             'specified wake_file. \n')
        if 'time' not in wake_file_columns:
            raise ValueError("No wake_file_column with name 'time' has "
                             'been specified. \n')
        for i, column_name in enumerate(wake_file_columns):
            self.wake_table[column_name] = wake_data[:, i]
        self.n_turns_wake = n_turns_wake

    def get_wake_kicks(self, slicer):
        """wakes.py:219-285."""
        from .wake_kicks import (ConstantWakeKickX, ConstantWakeKickY,
                                 DipoleWakeKickXY, DipoleWakeKickYX,
                                 QuadrupoleWakeKickXY, QuadrupoleWakeKickYX)
        n = self.n_turns_wake
        order = [('constant_x', ConstantWakeKickX),
                 ('constant_y', ConstantWakeKickY),
                 ('longitudinal', ConstantWakeKickZ),
                 ('dipole_x', DipoleWakeKickX),
                 ('dipole_y', DipoleWakeKickY),
                 ('dipole_xy', DipoleWakeKickXY),
                 ('dipole_yx', DipoleWakeKickYX),
                 ('quadrupole_x', QuadrupoleWakeKickX),
                 ('quadrupole_y', QuadrupoleWakeKickY),
                 ('quadrupole_xy', QuadrupoleWakeKickXY),
                 ('quadrupole_yx', QuadrupoleWakeKickYX)]
        kicks = []
        for name, cls in order:
            if not self._is_provided(name):
                continue
            wf = (self.function_longitudinal() if name == 'longitudinal'
                  else self.function_transverse(name))
            kicks.append(cls(wf, slicer, n))
        return kicks

    def _is_provided(self, wake_component):
        return wake_component in self.wake_table

    def function_transverse(self, wake_component):
        """wakes.py:298-339."""
        from scipy.interpolate import interp1d
        convert_to_s = 1e-9
        convert_to_V_per_Cm = 1e15
        time = convert_to_s * self.wake_table['time']
        wake_strength = -convert_to_V_per_Cm * self.wake_table[wake_component]
        interpolation_function = interp1d(time, wake_strength)
        if (time[0] == 0) and (wake_strength[0] == 0):
            def wake(dt, *args, **kwargs):
                dt = dt.clip(max=0)
                return interpolation_function(-dt)
            self.prints(wake_component + ' Assuming ultrarelativistic wake.')
        elif time[0] < 0:
            def wake(dt, *args, **kwargs):
                return interpolation_function(-dt)
            self.prints(wake_component + ' Found low beta wake.')
        else:
            raise ValueError(wake_component + ' does not meet requirements.')
        return wake

    def function_longitudinal(self):
        """wakes.py:341-376 (beam loading theorem: half the value at
        dt = 0 for tables starting at 0)."""
        from scipy.interpolate import interp1d
        convert_to_s = 1e-9
        convert_to_V_per_C = 1e12
        time = convert_to_s * self.wake_table['time']
        wake_strength = convert_to_V_per_C * self.wake_table['longitudinal']
        interpolation_function = interp1d(time, wake_strength,
                                          bounds_error=False, fill_value=0.)

        def wake(dt, *args, **kwargs):
            wake_interpolated = interpolation_function(-dt)
            if time[0] == 0:
                return (np.sign(-dt) + 1.) / 2. * wake_interpolated
            elif time[0] < 0:
                return wake_interpolated
            raise ValueError('Longitudinal wake component does not meet '
                             'requirements.')
        return wake
