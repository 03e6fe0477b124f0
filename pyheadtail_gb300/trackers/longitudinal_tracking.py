"""Longitudinal maps for the GPU turn loop.

Mirrors PyHEADTAIL's trackers/longitudinal_tracking.py: ``LongitudinalMap``
(:28-81, slippage factor), ``Drift`` (:84-111), ``Kick`` (:114-203),
``LongitudinalOneTurnMap`` (:255-277), ``RFSystems`` (:280-594, Verlet
drift-kick-drift with phase lock and transverse shrinking) and
``LinearMap`` (:667-759).  Every ``track(beam)`` evaluates its host scalars
with the reference formulas at that point of the sequence -- including the
``beam.p0 += p_increment`` setter of every kick (:202) -- and appends an op
to the beam's pending program; the per-particle arithmetic runs in the fused
kernel.  RFBucket-based queries (bucket, Q_s from the bucket) are host-side
set-up that is not part of this package.
"""
from abc import ABCMeta, abstractmethod

import numpy as np
from scipy.constants import c

from .. import _engine as E
from .. import _native as N
from ..general.element import Element
from ..particles.slicing import clean_slices


class LongitudinalMap(Element, metaclass=ABCMeta):
    """Base with the slippage factor eta (longitudinal_tracking.py:62-81)."""

    def __init__(self, alpha_array, *args, **kwargs):
        self.alpha_array = alpha_array

    @abstractmethod
    def track(self, beam):
        pass

    def eta(self, dp, gamma):
        eta = 0
        for i in range(len(self.alpha_array)):
            eta_func = getattr(self, '_eta' + str(i))
            eta += eta_func(self.alpha_array, gamma) * (dp ** i)
        return eta

    @staticmethod
    def _eta0(alpha_array, gamma):
        return alpha_array[0] - gamma**-2

    def _eta0_only(self, gamma):
        """eta for the fused kernel: the reference defines _eta0 only, so a
        longer alpha_array raises the reference's AttributeError here."""
        for i in range(1, len(self.alpha_array)):
            getattr(self, '_eta' + str(i))
        return self._eta0(self.alpha_array, gamma)


class Drift(LongitudinalMap):
    """z -> beta_ratio z - eta(dp) dp L (longitudinal_tracking.py:84-111)."""

    def __init__(self, alpha_array, length, shrinkage_p_increment=0, *args,
                 **kwargs):
        super(Drift, self).__init__(alpha_array, *args, **kwargs)
        self.length = length
        self.shrinkage_p_increment = shrinkage_p_increment

    def _op(self, beam):
        beta_ratio = 1 - self.shrinkage_p_increment / (beam.gamma**3 * beam.p0)
        eta0 = self._eta0_only(beam.gamma)
        flags = N.FLAG_SHRINK if beta_ratio != 1 else 0
        p = {0: float(beta_ratio), 1: float(eta0), 2: float(self.length)}
        eh, el = E.split_ff(eta0 * self.length)
        bh, bl = E.split_ff(beta_ratio)
        pf = {0: bh, 1: eh, 2: el, 3: bl}
        return E.Op(N.OP_DRIFT, flags, p, pf)

    @clean_slices
    def track(self, beam):
        beam._engine.enqueue(self._op(beam))


class Kick(LongitudinalMap):
    """RF kick of one cavity (longitudinal_tracking.py:114-203)."""

    def __init__(self, alpha_array, circumference, harmonic, voltage,
                 phi_offset=0, p_increment=0, D_x=0, D_y=0, *args, **kwargs):
        super(Kick, self).__init__(alpha_array, *args, **kwargs)
        self.circumference = circumference
        self.harmonic = harmonic
        self.voltage = voltage
        self.phi_offset = phi_offset
        self.p_increment = p_increment
        self._phi_lock = 0
        self.D_x = D_x
        self.D_y = D_y

    def _op(self, beam, dispersion=None):
        """The RF_KICK op; dispersion: True / False force the reference's
        track_with_dispersion / track_without_dispersion, None follows
        D_x, D_y as its track does (longitudinal_tracking.py:168-181)."""
        amplitude = np.abs(beam.charge) * self.voltage / (beam.beta * c)
        p0_old = beam.p0
        beam.p0 += self.p_increment
        p0_new = beam.p0
        flags = 0
        if (bool(self.D_x or self.D_y) if dispersion is None
                else dispersion):
            flags |= N.FLAG_DISPERSION
        if self.phi_offset != 0:
            flags |= N.FLAG_PHI_OFFSET
        if self._phi_lock != 0:
            flags |= N.FLAG_PHI_LOCK
        if self.p_increment != 0:
            flags |= N.FLAG_P_INC
        p = {0: float(self.harmonic), 1: 2 * np.pi,
             2: float(self.circumference), 3: float(self.phi_offset),
             4: float(self._phi_lock), 5: float(amplitude), 6: float(p0_old),
             7: float(self.p_increment), 8: float(p0_new),
             9: float(self.D_x), 10: float(self.D_y),
             11: 1. / float(self.circumference), 12: 1. / float(p0_new)}
        # precision form: phase in turns = z h / C + (offset + lock) / 2 pi
        turns_per_m = np.float64(self.harmonic) / self.circumference
        off = (self.phi_offset + self._phi_lock) / (2 * np.pi)
        off -= np.floor(off)
        hh, hl = E.split_ff(turns_per_m)
        oh, ol = E.split_ff(off)
        ah, al = E.split_ff(amplitude / p0_new)
        rh, rl = E.split_ff(p0_old / p0_new)
        pf = {0: hh, 1: hl, 2: oh, 3: ol, 4: ah, 5: rh,
              6: np.float32(self.p_increment / p0_new),
              8: np.float32(self.D_x), 9: np.float32(self.D_y),
              10: al, 11: rl}
        return E.Op(N.OP_RF_KICK, flags, p, pf)

    def track(self, beam):
        beam._engine.enqueue(self._op(beam))

    def track_with_dispersion(self, beam):
        """longitudinal_tracking.py:183-193."""
        beam._engine.enqueue(self._op(beam, dispersion=True))

    def track_without_dispersion(self, beam):
        """longitudinal_tracking.py:195-203."""
        beam._engine.enqueue(self._op(beam, dispersion=False))


class LongitudinalOneTurnMap(LongitudinalMap, metaclass=ABCMeta):

    def __init__(self, alpha_array, circumference, *args, **kwargs):
        super(LongitudinalOneTurnMap, self).__init__(alpha_array, *args,
                                                     **kwargs)
        self.circumference = circumference


class _ListProxy(object):
    """List view of one attribute of the kicks (general/utils.py:11-76)."""

    def __init__(self, kicks, attr):
        self._kicks, self._attr = kicks, attr

    def __getitem__(self, i):
        if isinstance(i, slice):
            return [getattr(k, self._attr) for k in self._kicks[i]]
        return getattr(self._kicks[i], self._attr)

    def __setitem__(self, i, v):
        if isinstance(i, slice):
            for k, vv in zip(self._kicks[i], v):
                setattr(k, self._attr, vv)
        else:
            setattr(self._kicks[i], self._attr, v)

    def __len__(self):
        return len(self._kicks)

    def __iter__(self):
        return (getattr(k, self._attr) for k in self._kicks)

    def __repr__(self):
        return repr(list(self))


class RFSystems(LongitudinalOneTurnMap):
    """Drift(C/2) -> RF kicks -> Drift(C/2) (longitudinal_tracking.py:280-594)."""

    def __init__(self, circumference, harmonic_list, voltage_list,
                 phi_offset_list, alpha_array, gamma_reference,
                 p_increment=0, phase_lock=True, shrink_transverse=True,
                 shrink_longitudinal=False, D_x=0, D_y=0, charge=None,
                 mass=None, *args, **kwargs):
        self.charge = charge
        self.mass = mass
        self.gamma = gamma_reference
        super(RFSystems, self).__init__(alpha_array, circumference, *args,
                                        **kwargs)
        if not len(harmonic_list) == len(voltage_list) == len(phi_offset_list):
            self.warns('Parameter lists for RFSystems do not have the same '
                       'length!')
        self._shrinking = shrink_longitudinal
        self._shrink_transverse = shrink_transverse
        self._kicks = [Kick(alpha_array, self.circumference, h, V, dphi,
                            D_x=D_x, D_y=D_y)
                       for h, V, dphi in zip(harmonic_list, voltage_list,
                                             phi_offset_list)]
        self._elements = ([Drift(alpha_array, 0.5 * self.circumference)] +
                          self._kicks +
                          [Drift(alpha_array, 0.5 * self.circumference)])
        self._accelerating_kick = self._kicks[0]
        self._shrinking_drift = self._elements[-1]
        self.p_increment = p_increment
        if phase_lock:
            self._phaselock(gamma_reference, charge)
        self._voltages = _ListProxy(self._kicks, 'voltage')
        self._harmonics = _ListProxy(self._kicks, 'harmonic')
        self._phi_offsets = _ListProxy(self._kicks, 'phi_offset')

    @property
    def voltages(self):
        return self._voltages

    @voltages.setter
    def voltages(self, value):
        self.voltages[:] = value

    @property
    def harmonics(self):
        return self._harmonics

    @harmonics.setter
    def harmonics(self, value):
        self.harmonics[:] = value

    @property
    def phi_offsets(self):
        return self._phi_offsets

    @phi_offsets.setter
    def phi_offsets(self, value):
        self.phi_offsets[:] = value

    @property
    def p_increment(self):
        return self._accelerating_kick.p_increment

    @p_increment.setter
    def p_increment(self, value):
        self._accelerating_kick.p_increment = value
        if self._shrinking:
            self._shrinking_drift.shrinkage_p_increment = value

    def pop_kick(self, index):
        if index == 0:
            raise ValueError('Cannot remove accelerating / fundamental kick, '
                             'remove_kick(0) is not accepted.')
        kick = self._kicks.pop(index)
        self._elements.remove(kick)
        return kick

    def phi_s(self, gamma, charge):
        """longitudinal_tracking.py:532-544."""
        beta = np.sqrt(1 - gamma**-2)
        V = self._accelerating_kick.voltage
        if self.p_increment == 0 and V == 0:
            return 0
        deltaE = self.p_increment * beta * c
        return np.arcsin(deltaE / (np.abs(charge) * V))

    def _phaselock(self, gamma, charge):
        acc = self._accelerating_kick
        for kick in (k for k in self._kicks if k is not acc):
            kick._phi_lock -= (kick.harmonic / acc.harmonic *
                               self.phi_s(gamma, charge))

    def track(self, beam):
        """track_transverse_shrinking / track_no_transverse_shrinking
        (longitudinal_tracking.py:556-580)."""
        betagamma_old = beam.betagamma
        for m in self._elements:
            m.track(beam)
        if self.p_increment and self._shrink_transverse:
            f = np.sqrt(betagamma_old / beam.betagamma)
            beam._engine.enqueue(E.Op(N.OP_SCALE_TRANS, 0, {0: float(f)},
                                      {0: np.float32(f)}))
        beam.clean_slices()

    def track_transverse_shrinking(self, beam):
        self.track(beam)

    def track_no_transverse_shrinking(self, beam):
        """The RF elements only, without the transverse adiabatic damping
        (longitudinal_tracking.py:576-580)."""
        for m in self._elements:
            m.track(beam)
        if self.p_increment:
            self.clean_buckets()
        beam.clean_slices()

    def clean_buckets(self):
        """longitudinal_tracking.py:525-530; no RFBucket is kept here, so
        there is nothing else to erase."""
        self._rfbuckets = {}

    # -- removed from the reference's interface: the same notices
    #    (longitudinal_tracking.py:595-648)
    @property
    def rfbucket(self):
        raise RuntimeError('Interface change: ' +
                           'Use the get_bucket(beam) method ' +
                           'to obtain a (constant) blueprint of the ' +
                           'current state of the ' +
                           'longitudinal RF configuration.')

    @property
    def kicks(self):
        raise RuntimeError('Interface change: ' +
                           'Use the voltages, harmonics or phi_offsets ' +
                           'lists of RFSystems to access the kick parameters.')

    @property
    def elements(self):
        raise RuntimeError('Interface change: ' +
                           'Use the voltages, harmonics or phi_offsets ' +
                           'lists of RFSystems to access the kick parameters.')

    @property
    def fundamental_kick(self):
        raise RuntimeError('Interface change: ' +
                           'Use the voltages, harmonics or phi_offsets ' +
                           'lists of RFSystems to access the kick parameters.')

    @property
    def accelerating_kick(self):
        raise RuntimeError('Interface change: ' +
                           'Use the first entries of the voltages, harmonics ' +
                           'or phi_offsets lists of RFSystems to access the ' +
                           'kick parameters.')

    def set_voltage_list(self, voltage_list):
        raise RuntimeError('Interface change: ' +
                           'Use the list RFSystems.voltages .')

    def set_harmonic_list(self, harmonic_list):
        raise RuntimeError('Interface change: ' +
                           'Use the list RFSystems.harmonics .')

    def set_phi_offset_list(self, phi_offset_list):
        raise RuntimeError('Interface change: ' +
                           'Use the list RFSystems.phi_offsets .')

    @property
    def Q_s(self):
        """Small-amplitude synchrotron tune of this RF system at its
        reference gamma: the formula of RFBucket.Q_s
        (trackers/rf_bucket.py:268-279), which RFSystems.Q_s
        (longitudinal_tracking.py:461-464) reads from its bucket."""
        gamma = self.gamma
        beta = np.sqrt(1 - gamma**-2)
        p0 = np.sqrt(gamma**2 - 1) * self.mass * c
        eta0 = self.alpha_array[0] - gamma**-2
        hV = sum([h * self.voltages[i] for i, h in enumerate(self.harmonics)])
        return np.sqrt(np.abs(self.charge) * np.abs(eta0) * hV /
                       (2 * np.pi * p0 * beta * c))

    def get_bucket(self, *args, **kwargs):
        raise NotImplementedError('RFBucket (separatrix, bucket-matched '
                                  'distributions) is host-side set-up of the '
                                  'reference; build it with PyHEADTAIL')


class LinearMap(LongitudinalOneTurnMap):
    """Linear synchrotron motion (longitudinal_tracking.py:667-759)."""

    def __init__(self, alpha_array, circumference, Q_s, D_x=0, D_y=0, *args,
                 **kwargs):
        super(LinearMap, self).__init__(alpha_array, circumference, *args,
                                        **kwargs)
        assert len(np.atleast_1d(Q_s)) == 1, 'Q_s can only have one entry!'
        self.Q_s = Q_s
        self.D_x = D_x
        self.D_y = D_y
        if len(alpha_array) > 1:
            self.warns('The higher orders in the given alpha_array are '
                       'manifestly neglected.')

    @property
    def Qs(self):
        """longitudinal_tracking.py:716-718."""
        return self.Q_s

    def _op(self, beam, dispersion=None):
        """The LINEAR_LONG op; dispersion as for Kick._op (D = 0 makes the
        reference's dispersion passes, :731-741, no-ops)."""
        omega_0 = 2 * np.pi * beam.beta * c / self.circumference
        omega_s = self.Q_s * omega_0
        dQ_s = 2 * np.pi * self.Q_s
        cosdQ_s = np.cos(dQ_s)
        sindQ_s = np.sin(dQ_s)
        longfac = self.eta(0, beam.gamma) * beam.beta * c / omega_s
        flags = N.FLAG_DISPERSION if (
            bool(self.D_x or self.D_y) if dispersion is None
            else dispersion) else 0
        p = {0: float(cosdQ_s), 1: float(sindQ_s), 2: float(longfac),
             3: float(self.D_x), 4: float(self.D_y), 5: 1. / float(longfac)}
        # precision form: float-float cos, longfac*sin and sin/longfac
        ch, cl = E.split_ff(cosdQ_s)
        ah, al = E.split_ff(longfac * sindQ_s)
        bh, bl = E.split_ff(sindQ_s / longfac)
        pf = {0: ch, 1: cl, 2: ah, 3: al, 4: np.float32(self.D_x),
              5: np.float32(self.D_y), 6: bh, 7: bl}
        return E.Op(N.OP_LINEAR_LONG, flags, p, pf)

    def track(self, beam):
        beam._engine.enqueue(self._op(beam))
        beam.clean_slices()

    def track_with_dispersion(self, beam):
        """longitudinal_tracking.py:731-741."""
        beam._engine.enqueue(self._op(beam, dispersion=True))
        beam.clean_slices()

    def track_without_dispersion(self, beam):
        """longitudinal_tracking.py:743-759."""
        beam._engine.enqueue(self._op(beam, dispersion=False))
        beam.clean_slices()
