"""CPU oracle for the single-bunch turn loop -- TEST INFRASTRUCTURE ONLY.

This module restates, in NumPy, the arithmetic of PyHEADTAIL v1.16.5's
per-turn single-bunch tracking loop:

    TransverseSegmentMap (+ Chromaticity, AmplitudeDetuning)
    -> RFSystems (Drift / Kick / Drift) or LinearMap
    -> UniformBinSlicer (bin index, per-slice counts and moments)
    -> WakeField / WakeKick (resonator, resistive wall, multi-turn history)

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py`` (its
``cpu_baseline`` leg and ``--impl reference`` arm) may import it, and only as
the checker or the timed CPU baseline.  The GB300 product path never calls it.

Every expression keeps the reference's operation order so that results are
bit-identical to the reference's NumPy/Cython path.  That claim is pinned by
``tests/test_oracle_golden.py`` against fixtures produced by running the
reference itself (``tests/golden/make_golden.py``), by the reference's own
instability tests replayed from its bunches and traces
(``tests/test_oracle_reswall.py``, ``tests/test_oracle_bb_resonator.py``)
and, where the reference's source tree is present, at the full size of the
1e7- and 5e7-macroparticle workloads
(``tests/golden/compare_full_size.py``).  Citations are ``path:line``
inside the PyHEADTAIL source tree.
"""
from collections import deque
from math import factorial

import numpy as np
from scipy.constants import c, e

# --------------------------------------------------------------------------
# Beam: coordinates + the reference's scalar property chain
# --------------------------------------------------------------------------


class Beam(object):
    """Six FP64 coordinate arrays plus the scalar state of ``Particles``.

    The gamma -> beta / betagamma / p0 chain and the p0 setter restate
    ``particles/particles.py:74-104``; ``id`` follows ``:55``.
    """

    COORDS = ('x', 'xp', 'y', 'yp', 'z', 'dp')

    def __init__(self, coords, particlenumber_per_mp, charge, mass,
                 circumference, gamma):
        n = len(coords['x'])
        self.macroparticlenumber = n
        self.particlenumber_per_mp = particlenumber_per_mp
        self.charge = charge
        self.mass = mass
        self.circumference = circumference
        self.gamma = gamma
        self.id = np.arange(1, n + 1, dtype=np.int32)
        for k in self.COORDS:
            setattr(self, k, np.array(coords[k], dtype=np.float64, copy=True))

    @property
    def gamma(self):
        return self._gamma

    @gamma.setter
    def gamma(self, value):
        # particles/particles.py:77-82
        self._gamma = value
        self._beta = np.sqrt(1 - self.gamma**-2)
        self._betagamma = np.sqrt(self.gamma**2 - 1)
        self._p0 = self.betagamma * self.mass * c

    @property
    def beta(self):
        return self._beta

    @property
    def betagamma(self):
        return self._betagamma

    @property
    def p0(self):
        return self._p0

    @p0.setter
    def p0(self, value):
        # particles/particles.py:101-103
        self.gamma = np.sqrt(1 + (value / (self.mass * c))**2)

    @property
    def charge_per_mp(self):
        return self.particlenumber_per_mp * self.charge

    @property
    def intensity(self):
        return self.particlenumber_per_mp * self.macroparticlenumber

    def copy(self):
        b = Beam({k: getattr(self, k) for k in self.COORDS},
                 self.particlenumber_per_mp, self.charge, self.mass,
                 self.circumference, self._gamma)
        return b

    def coords(self):
        return {k: getattr(self, k).copy() for k in self.COORDS}

    # bunch statistics: particles/particles.py:311-390 over pmath's CPU
    # table (general/pmath.py:183-189: np.mean and the stats.pyx functions)
    def mean_x(self):
        return np.mean(self.x)

    def mean_xp(self):
        return np.mean(self.xp)

    def mean_y(self):
        return np.mean(self.y)

    def mean_yp(self):
        return np.mean(self.yp)

    def mean_z(self):
        return np.mean(self.z)

    def mean_dp(self):
        return np.mean(self.dp)

    def sigma_x(self):
        return std(self.x)

    def sigma_y(self):
        return std(self.y)

    def sigma_z(self):
        return std(self.z)

    def sigma_xp(self):
        return std(self.xp)

    def sigma_yp(self):
        return std(self.yp)

    def sigma_dp(self):
        return std(self.dp)

    def effective_normalized_emittance_x(self):
        return emittance(self.x, self.xp, None) * self.betagamma

    def effective_normalized_emittance_y(self):
        return emittance(self.y, self.yp, None) * self.betagamma

    def effective_normalized_emittance_z(self):
        return 4 * np.pi * emittance(self.z, self.dp, None) * self.p0 / e

    def epsn_x(self):
        return emittance(self.x, self.xp, self.dp) * self.betagamma

    def epsn_y(self):
        return emittance(self.y, self.yp, self.dp) * self.betagamma

    def epsn_z(self):
        return self.effective_normalized_emittance_z()

    def dispersion_x(self):
        return dispersion(self.x, self.dp)

    def dispersion_y(self):
        return dispersion(self.y, self.dp)

    def alpha_Twiss_x(self):
        return get_alpha(self.x, self.xp, self.dp)

    def alpha_Twiss_y(self):
        return get_alpha(self.y, self.yp, self.dp)

    def beta_Twiss_x(self):
        return get_beta(self.x, self.xp, self.dp)

    def beta_Twiss_y(self):
        return get_beta(self.y, self.yp, self.dp)

    def gamma_Twiss_x(self):
        return get_gamma(self.x, self.xp, self.dp)

    def gamma_Twiss_y(self):
        return get_gamma(self.y, self.yp, self.dp)


def cov_shifted(a, b):
    """Shifted single-pass covariance, ``cobra_functions/stats.pyx:17-45``."""
    n = a.shape[0]
    if n < 2:
        return 0.
    sa = a[0]
    sb = b[0]
    da = a - sa
    db = b - sb
    # the Cython loop sums sequentially; np.add.accumulate keeps that order
    a_sum = np.add.accumulate(da)[-1]
    b_sum = np.add.accumulate(db)[-1]
    ab_sum = np.add.accumulate(da * db)[-1]
    return (ab_sum - a_sum * b_sum / n) / (n - 1)


def std(u):
    """stats.pyx:49-54."""
    return np.sqrt(cov_shifted(u, u))


def dispersion(u, dp):
    """stats.pyx:57-70: <u dp> / <dp^2> (0 when <dp^2> is 0)."""
    mean_u_dp = np.mean(np.multiply(u, dp))
    mean_dp2 = np.mean(np.multiply(dp, dp))
    if mean_dp2 > 0:
        return mean_u_dp / mean_dp2
    return 0


def emittance(u, up, dp):
    """stats.pyx:73-122: sqrt of the determinant of the beam matrix with
    the dispersive parts removed (none when dp is None or constant)."""
    cov_u2 = cov_shifted(u, u)
    cov_up2 = cov_shifted(up, up)
    cov_u_up = cov_shifted(up, u)
    term_u2_dp = term_u_up_dp = term_up2_dp = 0.
    if dp is not None:
        cov_dp2 = cov_shifted(dp, dp)
        if cov_dp2 != 0:
            cov_u_dp = cov_shifted(u, dp)
            cov_up_dp = cov_shifted(up, dp)
            term_u2_dp = cov_u_dp * cov_u_dp / cov_dp2
            term_u_up_dp = cov_u_dp * cov_up_dp / cov_dp2
            term_up2_dp = cov_up_dp * cov_up_dp / cov_dp2
    sigma11 = cov_u2 - term_u2_dp
    sigma12 = cov_u_up - term_u_up_dp
    sigma22 = cov_up2 - term_up2_dp
    return np.sqrt(sigma11 * sigma22 - sigma12 * sigma12)


def get_alpha(u, up, dp):
    """stats.pyx:126-145."""
    cov_u_up = cov_shifted(u, up)
    cov_dp2, cov_u_dp, cov_up_dp = 1., 0., 0.
    if dp is not None:
        cov_dp2 = cov_shifted(dp, dp)
        cov_u_dp = cov_shifted(u, dp)
        cov_up_dp = cov_shifted(up, dp)
    sigma12 = cov_u_up - cov_u_dp * cov_up_dp / cov_dp2
    return -sigma12 / emittance(u, up, dp)


def get_beta(u, up, dp):
    """stats.pyx:148-165."""
    cov_u2 = cov_shifted(u, u)
    cov_u_dp, cov_dp2 = 0., 1.
    if dp is not None:
        cov_u_dp = cov_shifted(u, dp)
        cov_dp2 = cov_shifted(dp, dp)
    sigma11 = cov_u2 - cov_u_dp * cov_u_dp / cov_dp2
    return sigma11 / emittance(u, up, dp)


def get_gamma(u, up, dp):
    """stats.pyx:168-185."""
    cov_up2 = cov_shifted(up, up)
    cov_up_dp, cov_dp2 = 0., 1.
    if dp is not None:
        cov_up_dp = cov_shifted(up, dp)
        cov_dp2 = cov_shifted(dp, dp)
    sigma22 = cov_up2 - cov_up_dp * cov_up_dp / cov_dp2
    return sigma22 / emittance(u, up, dp)


# --------------------------------------------------------------------------
# Transverse: trackers/transverse_tracking.py, trackers/detuners.py
# --------------------------------------------------------------------------


def segment_IJ(alpha_x_s0, beta_x_s0, alpha_x_s1, beta_x_s1,
               alpha_y_s0, beta_y_s0, alpha_y_s1, beta_y_s1):
    """I (cosine) and J (sine) matrices, transverse_tracking.py:71-103."""
    I = np.zeros((4, 4))
    J = np.zeros((4, 4))
    I[0, 0] = np.sqrt(beta_x_s1 / beta_x_s0)
    I[1, 0] = (np.sqrt(1. / (beta_x_s0 * beta_x_s1)) *
               (alpha_x_s0 - alpha_x_s1))
    I[1, 1] = np.sqrt(beta_x_s0 / beta_x_s1)
    I[2, 2] = np.sqrt(beta_y_s1 / beta_y_s0)
    I[3, 2] = (np.sqrt(1. / (beta_y_s0 * beta_y_s1)) *
               (alpha_y_s0 - alpha_y_s1))
    I[3, 3] = np.sqrt(beta_y_s0 / beta_y_s1)
    J[0, 0] = np.sqrt(beta_x_s1 / beta_x_s0) * alpha_x_s0
    J[0, 1] = np.sqrt(beta_x_s0 * beta_x_s1)
    J[1, 0] = -(np.sqrt(1. / (beta_x_s0 * beta_x_s1)) *
                (1. + alpha_x_s0 * alpha_x_s1))
    J[1, 1] = -np.sqrt(beta_x_s0 / beta_x_s1) * alpha_x_s1
    J[2, 2] = np.sqrt(beta_y_s1 / beta_y_s0) * alpha_y_s0
    J[2, 3] = np.sqrt(beta_y_s0 * beta_y_s1)
    J[3, 2] = -(np.sqrt(1. / (beta_y_s0 * beta_y_s1)) *
                (1. + alpha_y_s0 * alpha_y_s1))
    J[3, 3] = -np.sqrt(beta_y_s0 / beta_y_s1) * alpha_y_s1
    return I, J


class ChromaDetuner(object):
    """ChromaticitySegment, detuners.py:48-98 (Horner forms :85-97)."""

    def __init__(self, dQp_x, dQp_y):
        self.cx = [q / float(factorial(i + 1))
                   for i, q in enumerate(np.atleast_1d(dQp_x))]
        self.cy = [q / float(factorial(i + 1))
                   for i, q in enumerate(np.atleast_1d(dQp_y))]

    @staticmethod
    def _poly(coeffs, dp):
        n = len(coeffs)
        if n == 1:
            return coeffs[0] * dp
        if n == 2:
            return (coeffs[0] + coeffs[1] * dp) * dp
        if n == 3:
            return (coeffs[0] + (coeffs[1] + coeffs[2] * dp) * dp) * dp
        # order > 3: detuners.py:95-97 prepends a zero on *every* call
        coeffs.insert(0, 0)
        return np.polynomial.polynomial.polyval(dp, coeffs)

    def detune(self, beam):
        return self._poly(self.cx, beam.dp), self._poly(self.cy, beam.dp)


class AmplitudeDetuner(object):
    """AmplitudeDetuningSegment.detune, detuners.py:101-151."""

    def __init__(self, dapp_x, dapp_y, dapp_xy, dapp_yx,
                 alpha_x, beta_x, alpha_y, beta_y):
        self.dapp_x, self.dapp_y = dapp_x, dapp_y
        self.dapp_xy, self.dapp_yx = dapp_xy, dapp_yx
        self.alpha_x, self.beta_x = alpha_x, beta_x
        self.alpha_y, self.beta_y = alpha_y, beta_y

    def detune(self, beam):
        Jx = 1 / 2 * (
            (1 + self.alpha_x**2) / self.beta_x * beam.x**2
            + 2 * self.alpha_x * beam.x * beam.xp
            + self.beta_x * beam.xp**2)
        Jy = 1 / 2 * (
            (1 + self.alpha_y**2) / self.beta_y * beam.y**2
            + 2 * self.alpha_y * beam.y * beam.yp
            + self.beta_y * beam.yp**2)
        dQ_x = (self.dapp_x * Jx + self.dapp_xy * Jy) / beam.p0
        dQ_y = (self.dapp_y * Jy + self.dapp_yx * Jx) / beam.p0
        return dQ_x, dQ_y


class TransverseSegment(object):
    """TransverseSegmentMap.track, transverse_tracking.py:138-196."""

    def __init__(self, alpha_x_s0, beta_x_s0, D_x_s0, alpha_x_s1, beta_x_s1,
                 D_x_s1, alpha_y_s0, beta_y_s0, D_y_s0, alpha_y_s1, beta_y_s1,
                 D_y_s1, dQ_x, dQ_y, detuners=()):
        self.D = (D_x_s0, D_x_s1, D_y_s0, D_y_s1)
        self.dQ_x, self.dQ_y = dQ_x, dQ_y
        self.I, self.J = segment_IJ(alpha_x_s0, beta_x_s0, alpha_x_s1,
                                    beta_x_s1, alpha_y_s0, beta_y_s0,
                                    alpha_y_s1, beta_y_s1)
        self.detuners = list(detuners)
        # transverse_tracking.py:65-69
        self.with_dispersion = not np.allclose(list(self.D), np.zeros(4),
                                               atol=1e-3)

    def track(self, beam):
        dphi_x = self.dQ_x
        dphi_y = self.dQ_y
        is_array = False
        for d in self.detuners:
            ddx, ddy = d.detune(beam)
            dphi_x += ddx
            dphi_y += ddy
            is_array = True
        dphi_x *= 2. * np.pi
        dphi_y *= 2. * np.pi
        if is_array:
            dphi_x = np.atleast_1d(dphi_x)
            dphi_y = np.atleast_1d(dphi_y)
            s_x, c_x = np.sin(dphi_x), np.cos(dphi_x)
            s_y, c_y = np.sin(dphi_y), np.cos(dphi_y)
        else:
            c_x, c_y = np.cos(dphi_x), np.cos(dphi_y)
            s_x, s_y = np.sin(dphi_x), np.sin(dphi_y)
        I, J = self.I, self.J
        M00 = I[0, 0] * c_x + J[0, 0] * s_x
        M01 = I[0, 1] * c_x + J[0, 1] * s_x
        M10 = I[1, 0] * c_x + J[1, 0] * s_x
        M11 = I[1, 1] * c_x + J[1, 1] * s_x
        M22 = I[2, 2] * c_y + J[2, 2] * s_y
        M23 = I[2, 3] * c_y + J[2, 3] * s_y
        M32 = I[3, 2] * c_y + J[3, 2] * s_y
        M33 = I[3, 3] * c_y + J[3, 3] * s_y
        if self.with_dispersion:
            beam.x -= self.D[0] * beam.dp
            beam.y -= self.D[2] * beam.dp
        beam.x, beam.xp = M00 * beam.x + M01 * beam.xp, M10 * beam.x + M11 * beam.xp
        beam.y, beam.yp = M22 * beam.y + M23 * beam.yp, M32 * beam.y + M33 * beam.yp
        if self.with_dispersion:
            beam.x += self.D[1] * beam.dp
            beam.y += self.D[3] * beam.dp


def transverse_map(s, alpha_x, beta_x, D_x, alpha_y, beta_y, D_y,
                   accQ_x, accQ_y, chroma=None, amplitude=None,
                   detuner_order=('chroma', 'amplitude')):
    """TransverseMap._generate_segment_maps, transverse_tracking.py:275-329.

    ``chroma`` = (Qp_x, Qp_y) (detuners.py:283-312); ``amplitude`` =
    (app_x, app_y, app_xy) (detuners.py:201-281).
    """
    s = np.asarray(s, dtype=float)
    seg_len = np.diff(s) / s[-1]
    dQ_x = accQ_x * seg_len if np.ndim(accQ_x) == 0 else np.diff(accQ_x)
    dQ_y = accQ_y * seg_len if np.ndim(accQ_y) == 0 else np.diff(accQ_y)
    n_seg = len(s) - 1
    dmu_x = dQ_x / np.atleast_1d(accQ_x)[-1]
    dmu_y = dQ_y / np.atleast_1d(accQ_y)[-1]
    segs = []
    for seg in range(n_seg):
        s0 = seg % n_seg
        s1 = (seg + 1) % n_seg
        dets = []
        for kind in detuner_order:
            if kind == 'chroma' and chroma is not None:
                Qp_x, Qp_y = np.atleast_1d(chroma[0]), np.atleast_1d(chroma[1])
                dets.append(ChromaDetuner([q * dmu_x[s0] for q in Qp_x],
                                          [q * dmu_y[s0] for q in Qp_y]))
            elif kind == 'amplitude' and amplitude is not None:
                app_x, app_y, app_xy = amplitude
                dets.append(AmplitudeDetuner(
                    app_x * dmu_x[s0], app_y * dmu_y[s0],
                    app_xy * dmu_x[s0], app_xy * dmu_y[s0],
                    alpha_x[s0], beta_x[s0], alpha_y[s0], beta_y[s0]))
        segs.append(TransverseSegment(
            alpha_x[s0], beta_x[s0], D_x[s0], alpha_x[s1], beta_x[s1], D_x[s1],
            alpha_y[s0], beta_y[s0], D_y[s0], alpha_y[s1], beta_y[s1], D_y[s1],
            dQ_x[seg], dQ_y[seg], dets))
    return segs


# --------------------------------------------------------------------------
# Longitudinal: trackers/longitudinal_tracking.py
# --------------------------------------------------------------------------


def eta(alpha_array, dp, gamma):
    """LongitudinalMap.eta, longitudinal_tracking.py:62-81 (only _eta0
    exists in the reference, so alpha arrays longer than 1 raise there)."""
    out = 0
    for i in range(len(alpha_array)):
        if i > 0:
            raise AttributeError("'Drift' object has no attribute '_eta%d'" % i)
        eta_i = alpha_array[0] - gamma**-2
        out += eta_i * (dp ** i)
    return out


class Drift(object):
    """longitudinal_tracking.py:84-111."""

    def __init__(self, alpha_array, length, shrinkage_p_increment=0):
        self.alpha_array = alpha_array
        self.length = length
        self.shrinkage_p_increment = shrinkage_p_increment

    def track(self, beam):
        beta_ratio = 1 - self.shrinkage_p_increment / (beam.gamma**3 * beam.p0)
        beam.z = (beta_ratio * beam.z -
                  eta(self.alpha_array, beam.dp, beam.gamma) * beam.dp *
                  self.length)


class Kick(object):
    """longitudinal_tracking.py:114-203."""

    def __init__(self, alpha_array, circumference, harmonic, voltage,
                 phi_offset=0, p_increment=0, D_x=0, D_y=0):
        self.circumference = circumference
        self.harmonic = harmonic
        self.voltage = voltage
        self.phi_offset = phi_offset
        self.p_increment = p_increment
        self._phi_lock = 0
        self.D_x, self.D_y = D_x, D_y

    def track(self, beam):
        if not self.D_x and not self.D_y:
            return self._track_plain(beam)
        beam.x -= self.D_x * beam.dp
        beam.y -= self.D_y * beam.dp
        self._track_plain(beam)
        beam.x += self.D_x * beam.dp
        beam.y += self.D_y * beam.dp

    def _track_plain(self, beam):
        amplitude = np.abs(beam.charge) * self.voltage / (beam.beta * c)
        phi = (self.harmonic * (2 * np.pi * beam.z / self.circumference)
               + self.phi_offset + self._phi_lock)
        delta_p = beam.dp * beam.p0
        delta_p += amplitude * np.sin(phi) - self.p_increment
        beam.p0 += self.p_increment
        beam.dp = delta_p / beam.p0


class RFSystems(object):
    """RFSystems, longitudinal_tracking.py:280-594 (Verlet drift-kick-drift,
    phase lock :582-593, transverse shrinking :546-574)."""

    def __init__(self, circumference, harmonic_list, voltage_list,
                 phi_offset_list, alpha_array, gamma_reference, p_increment=0,
                 phase_lock=True, shrink_transverse=True,
                 shrink_longitudinal=False, D_x=0, D_y=0, charge=None,
                 mass=None):
        self.alpha_array = alpha_array
        self.circumference = circumference
        self._shrinking = shrink_longitudinal
        self.shrink_transverse = shrink_transverse
        self._kicks = [Kick(alpha_array, circumference, h, V, dphi,
                            D_x=D_x, D_y=D_y)
                       for h, V, dphi in zip(harmonic_list, voltage_list,
                                             phi_offset_list)]
        self._elements = ([Drift(alpha_array, 0.5 * circumference)] +
                          self._kicks +
                          [Drift(alpha_array, 0.5 * circumference)])
        self.p_increment = p_increment
        if phase_lock:
            acc = self._kicks[0]
            for k in self._kicks[1:]:
                k._phi_lock -= (k.harmonic / acc.harmonic *
                                self.phi_s(gamma_reference, charge))

    @property
    def p_increment(self):
        return self._kicks[0].p_increment

    @p_increment.setter
    def p_increment(self, value):
        self._kicks[0].p_increment = value
        if self._shrinking:
            self._elements[-1].shrinkage_p_increment = value

    def phi_s(self, gamma, charge):
        beta = np.sqrt(1 - gamma**-2)
        V = self._kicks[0].voltage
        if self.p_increment == 0 and V == 0:
            return 0
        deltaE = self.p_increment * beta * c
        return np.arcsin(deltaE / (np.abs(charge) * V))

    def track(self, beam):
        betagamma_old = beam.betagamma
        for m in self._elements:
            m.track(beam)
        if self.p_increment and self.shrink_transverse:
            f = np.sqrt(betagamma_old / beam.betagamma)
            beam.x *= f
            beam.xp *= f
            beam.y *= f
            beam.yp *= f


class LinearMap(object):
    """LinearMap, longitudinal_tracking.py:667-759 (always entered through
    track_with_dispersion, :720-741)."""

    def __init__(self, alpha_array, circumference, Q_s, D_x=0, D_y=0):
        self.alpha_array = alpha_array
        self.circumference = circumference
        self.Q_s = Q_s
        self.D_x, self.D_y = D_x, D_y

    def track(self, beam):
        beam.x -= self.D_x * beam.dp
        beam.y -= self.D_y * beam.dp
        omega_0 = 2 * np.pi * beam.beta * c / self.circumference
        omega_s = self.Q_s * omega_0
        dQ_s = 2 * np.pi * self.Q_s
        cosdQ_s = np.cos(dQ_s)
        sindQ_s = np.sin(dQ_s)
        z0 = beam.z
        dp0 = beam.dp
        longfac = eta(self.alpha_array, 0, beam.gamma) * beam.beta * c / omega_s
        beam.z = z0 * cosdQ_s - longfac * dp0 * sindQ_s
        beam.dp = dp0 * cosdQ_s + z0 / longfac * sindQ_s
        beam.x += self.D_x * beam.dp
        beam.y += self.D_y * beam.dp


# --------------------------------------------------------------------------
# Slicing: particles/slicing.py, cobra_functions/stats.pyx
# --------------------------------------------------------------------------


class SliceSet(object):
    """particles/slicing.py:58-317 (the attributes the hot path reads)."""

    def __init__(self, z_bins, idx, beam):
        self.z_bins = z_bins
        self.slice_index_of_particle = idx
        self.n_slices = len(z_bins) - 1
        # Slicer.extract_beam_parameters, slicing.py:384-393
        self.beta = beam.beta
        self.gamma = beam.gamma
        self.p0 = beam.p0
        self.age = 0
        within = (idx < self.n_slices) & (idx >= 0)
        # pmath.py:200-203
        self.particles_within_cuts = np.where(within)[0].astype(np.int32)
        # stats.pyx:192-202 (sequential count == bincount)
        s_idx = idx[self.particles_within_cuts]
        self.n_macroparticles_per_slice = np.bincount(
            s_idx, minlength=self.n_slices).astype(np.int32)

    @property
    def z_centers(self):
        return self.z_bins[:-1] + 0.5 * (self.z_bins[1:] - self.z_bins[:-1])

    def convert_to_time(self, z):
        return z / (self.beta * c)

    def mean_per_slice(self, u):
        """stats.pyx:235-253: sequential sum in particle order, then divide
        non-empty slices by their count.  bincount accumulates in the same
        index order."""
        p = self.particles_within_cuts
        sums = np.bincount(self.slice_index_of_particle[p], weights=u[p],
                           minlength=self.n_slices)
        n = self.n_macroparticles_per_slice
        out = np.zeros(self.n_slices)
        nz = n != 0
        out[nz] = sums[nz] / n[nz]
        return out

    def cov_per_slice(self, a, b):
        """stats.pyx:290-319 (two-pass, n-1 normalisation)."""
        p = self.particles_within_cuts
        s = self.slice_index_of_particle[p]
        ma = self.mean_per_slice(a)
        mb = self.mean_per_slice(b)
        acc = np.bincount(s, weights=(a[p] - ma[s]) * (b[p] - mb[s]),
                          minlength=self.n_slices)
        n = self.n_macroparticles_per_slice
        big = n > 1
        acc[big] = acc[big] / (n[big] - 1)
        return acc

    def std_per_slice(self, u):
        """stats.pyx:258-286."""
        p = self.particles_within_cuts
        s = self.slice_index_of_particle[p]
        mu = self.mean_per_slice(u)
        du = u[p] - mu[s]
        acc = np.bincount(s, weights=du * du, minlength=self.n_slices)
        n = self.n_macroparticles_per_slice
        big = n > 1
        acc[big] = acc[big] / (n[big] - 1)
        return np.sqrt(acc)

    def emittance_per_slice(self, u, up, dp=None):
        """stats.pyx:374-425 (uses _det_beam_matrix, :71-80)."""
        cu2 = self.cov_per_slice(u, u)
        cuup = self.cov_per_slice(u, up)
        cup2 = self.cov_per_slice(up, up)
        if dp is not None:
            cudp = self.cov_per_slice(u, dp)
            cupdp = self.cov_per_slice(up, dp)
            cdp2 = self.cov_per_slice(dp, dp)
        n = self.n_macroparticles_per_slice
        out = np.zeros(self.n_slices)
        for i in range(self.n_slices):
            if n[i] > 1:
                s11, s12, s22 = cu2[i], cuup[i], cup2[i]
                if dp is not None and cdp2[i] != 0.:
                    s11 -= cudp[i] * cudp[i] / cdp2[i]
                    s12 -= cudp[i] * cupdp[i] / cdp2[i]
                    s22 -= cupdp[i] * cupdp[i] / cdp2[i]
                out[i] = np.sqrt(s11 * s22 - s12 * s12)
        return out


class UniformBinSlicer(object):
    """UniformBinSlicer, particles/slicing.py:532-615 (cuts :395-413)."""

    mode = 'uniform_bin'

    def __init__(self, n_slices, n_sigma_z=None, z_cuts=None):
        self.n_slices = n_slices
        self.n_sigma_z = n_sigma_z
        self.z_cuts = z_cuts

    def get_long_cuts(self, beam):
        if self.z_cuts is not None:
            return self.z_cuts
        elif self.n_sigma_z:
            tail = beam.mean_z() - self.n_sigma_z * beam.sigma_z()
            head = beam.mean_z() + self.n_sigma_z * beam.sigma_z()
        else:
            tail = np.min(beam.z)
            head = np.max(beam.z)
            head += abs(head) * 1e-15
        return tail, head

    def bins_and_index(self, beam):
        """compute_sliceset_kwargs, slicing.py:599-615."""
        tail, head = self.get_long_cuts(beam)
        width = (head - tail) / float(self.n_slices)
        z_bins = np.arange(tail, head + 1e-7 * width, width, dtype=np.float64)
        idx = np.floor((beam.z - tail) / width).astype(np.int32)
        return z_bins, idx

    def slice(self, beam, statistics=()):
        z_bins, idx = self.bins_and_index(beam)
        ss = SliceSet(z_bins, idx, beam)
        for st in statistics:
            if st.startswith('mean_'):
                setattr(ss, st, ss.mean_per_slice(getattr(beam, st[5:])))
            elif st.startswith('sigma_'):
                setattr(ss, st, ss.std_per_slice(getattr(beam, st[6:])))
            elif st in ('epsn_x', 'epsn_y'):
                u = st[-1]
                setattr(ss, st, ss.emittance_per_slice(
                    getattr(beam, u), getattr(beam, u + 'p'), beam.dp) *
                    beam.betagamma)
            elif st in ('eff_epsn_x', 'eff_epsn_y'):
                u = st[-1]
                setattr(ss, st, ss.emittance_per_slice(
                    getattr(beam, u), getattr(beam, u + 'p'), None) *
                    beam.betagamma)
            elif st == 'epsn_z':
                setattr(ss, st, 4. * np.pi * ss.emittance_per_slice(
                    beam.z, beam.dp, None) * beam.p0 / e)
            else:
                raise ValueError(st)
        return ss


# --------------------------------------------------------------------------
# Wakes: impedances/wakes.py, impedances/wake_kicks.py
# --------------------------------------------------------------------------


class UniformChargeSlicer(UniformBinSlicer):
    """UniformChargeSlicer, particles/slicing.py:618-686: the bunch sorted
    by z is cut into slices of equal particle count (the remainder of the
    division goes to slices drawn with Python's random.sample); edges are
    the midpoints between the last particle of a slice and the first of the
    next; particles outside the cuts get index -1."""

    mode = 'uniform_charge'

    def bins_and_index(self, beam):
        from random import sample
        tail, head = self.get_long_cuts(beam)
        S = self.n_slices
        n = len(beam.z)
        order = np.argsort(beam.z)
        z_sorted = beam.z.take(order)
        below_tail = np.searchsorted(z_sorted, tail)
        from_head = n - np.searchsorted(z_sorted, head)
        inside = n - below_tail - from_head
        extra = sample(list(range(S)), inside % S)
        per_slice = (inside // S) * np.ones(S, dtype=np.int32)
        per_slice[extra] += 1
        bounds = np.cumsum(np.hstack((below_tail, per_slice, from_head)),
                           dtype=np.int32)[:-1]
        z_bins = np.empty(S + 1)
        z_bins[1:-1] = (z_sorted[bounds[1:-1] - 1] + z_sorted[bounds[1:-1]]) / 2
        z_bins[0], z_bins[-1] = tail, head
        idx_sorted = -np.ones(n, dtype=np.int32)
        for k in range(S):
            idx_sorted[bounds[k]:bounds[k + 1]] = k
        idx = np.empty(n, dtype=np.int32)
        np.put(idx, np.arange(n).take(order), idx_sorted)
        return z_bins, idx


def resonator_transverse(R_shunt, frequency, Q, yokoya):
    """Resonator.function_transverse, wakes.py:450-470."""
    omega = 2 * np.pi * frequency
    alpha = omega / (2 * Q)
    omegabar = np.sqrt(np.abs(omega**2 - alpha**2))

    def wake(dt, *args, **kwargs):
        dt = dt.clip(max=0)
        if Q > 0.5:
            y = (yokoya * R_shunt * omega**2 / (Q * omegabar) *
                 np.exp(alpha * dt) * np.sin(omegabar * dt))
        elif Q == 0.5:
            y = (yokoya * R_shunt * omega**2 / Q * np.exp(alpha * dt) * dt)
        else:
            y = (yokoya * R_shunt * omega**2 / (Q * omegabar) *
                 np.exp(alpha * dt) * np.sinh(omegabar * dt))
        return y
    return wake


def resonator_longitudinal(R_shunt, frequency, Q):
    """Resonator.function_longitudinal, wakes.py:472-493."""
    omega = 2 * np.pi * frequency
    alpha = omega / (2 * Q)
    omegabar = np.sqrt(np.abs(omega**2 - alpha**2))

    def wake(dt, *args, **kwargs):
        if Q > 0.5:
            y = (-(np.sign(dt) - 1) * R_shunt * alpha * np.exp(alpha * dt) *
                 (np.cos(omegabar * dt) + alpha / omegabar *
                  np.sin(omegabar * dt)))
        elif Q == 0.5:
            y = (-(np.sign(dt) - 1) * R_shunt * alpha * np.exp(alpha * dt) *
                 (1. + alpha * dt))
        else:
            y = (-(np.sign(dt) - 1) * R_shunt * alpha * np.exp(alpha * dt) *
                 (np.cosh(omegabar * dt) + alpha / omegabar *
                  np.sinh(omegabar * dt)))
        return y
    return wake


def resistive_wall_transverse(pipe_radius, length, conductivity, dt_min,
                              yokoya):
    """ResistiveWall.function_transverse, wakes.py:611-624."""
    mu_r = 1
    Z_0 = 119.9169832 * np.pi
    pipe_radius = np.array([pipe_radius]).flatten()

    def wake(dt, *args, **kwargs):
        y = (yokoya * (np.sign(dt + np.abs(dt_min)) - 1) / 2. *
             np.sqrt(kwargs['beta']) * length / np.pi /
             pipe_radius**3 * np.sqrt(-mu_r / np.pi /
             conductivity / dt.clip(max=-abs(dt_min)))) * np.sqrt(Z_0 * c)
        return y
    return wake


class TransverseDamper(object):
    """Ideal transverse damper, feedback/transverse_damper.py:17-86."""

    def __init__(self, dampingrate_x, dampingrate_y, phase=90,
                 local_beta_function=None):
        self.gain_x = 2 / dampingrate_x if dampingrate_x else None
        self.gain_y = 2 / dampingrate_y if dampingrate_y else None
        self.phase_in_2pi = phase / 360. * 2 * np.pi
        self.local_beta_function = local_beta_function

    def track(self, beam):
        # track_all's order (:77-86); one plane: track_horizontal/_vertical
        if self.gain_x is not None:
            beam.xp -= self.gain_x * np.sin(self.phase_in_2pi) * beam.mean_xp()
        if self.gain_y is not None:
            beam.yp -= self.gain_y * np.sin(self.phase_in_2pi) * beam.mean_yp()
        if self.local_beta_function:
            if self.gain_x is not None:
                beam.xp -= (self.gain_x * np.cos(self.phase_in_2pi) *
                            beam.mean_x() / self.local_beta_function)
            if self.gain_y is not None:
                beam.yp -= (self.gain_y * np.cos(self.phase_in_2pi) *
                            beam.mean_y() / self.local_beta_function)


def load_wake_table(wake_file, wake_file_columns):
    """WakeTable.__init__, impedances/wakes.py:201-217: columns by name."""
    data = np.loadtxt(wake_file)
    if len(wake_file_columns) != data.shape[1]:
        raise ValueError('wake_file_columns does not match the table')
    return {name: data[:, i] for i, name in enumerate(wake_file_columns)}


def table_transverse(table, component):
    """WakeTable.function_transverse, wakes.py:298-339: linear
    interpolation (scipy interp1d) of the table in SI units with the
    HEADTAIL sign; ultrarelativistic tables clip dt to <= 0."""
    from scipy.interpolate import interp1d
    time = 1e-9 * table['time']
    strength = -1e15 * table[component]
    f = interp1d(time, strength)
    if time[0] == 0 and strength[0] == 0:
        def wake(dt, *args, **kwargs):
            return f(-dt.clip(max=0))
    elif time[0] < 0:
        def wake(dt, *args, **kwargs):
            return f(-dt)
    else:
        raise ValueError(component + ' does not meet requirements.')
    return wake


def table_longitudinal(table):
    """WakeTable.function_longitudinal, wakes.py:341-376."""
    from scipy.interpolate import interp1d
    time = 1e-9 * table['time']
    strength = 1e12 * table['longitudinal']
    f = interp1d(time, strength, bounds_error=False, fill_value=0.)

    def wake(dt, *args, **kwargs):
        w = f(-dt)
        if time[0] == 0:
            return (np.sign(-dt) + 1.) / 2. * w
        if time[0] < 0:
            return w
        raise ValueError('longitudinal component does not meet requirements')
    return wake


# WakeTable.get_wake_kicks order (wakes.py:219-285): component, target,
# moment (None: count), quadrupolar coordinate
TABLE_KICKS = [('constant_x', 'xp', None, None), ('constant_y', 'yp', None, None),
               ('longitudinal', 'dp', None, None),
               ('dipole_x', 'xp', 'x', None), ('dipole_y', 'yp', 'y', None),
               ('dipole_xy', 'xp', 'y', None), ('dipole_yx', 'yp', 'x', None),
               ('quadrupole_x', 'xp', None, 'x'), ('quadrupole_y', 'yp', None, 'y'),
               ('quadrupole_xy', 'xp', None, 'y'),
               ('quadrupole_yx', 'yp', None, 'x')]


class WakeKick(object):
    """WakeKick base + dipole/quadrupole/constant kicks,
    wake_kicks.py:19-139, 144-361.

    ``target``: 'xp'/'yp'/'dp'; ``moment``: 'x', 'y' or None (count only);
    ``quad``: multiply by the particle's 'x'/'y' (quadrupolar kicks).
    """

    def __init__(self, wake_function, slicer, n_turns_wake, target, moment,
                 quad=None):
        self.wake_function = wake_function
        self.n_turns_wake = n_turns_wake
        self.target, self.moment, self.quad = target, moment, quad
        # wake_kicks.py:41-45
        if slicer.mode == 'uniform_bin' and (n_turns_wake == 1 or
                                             slicer.z_cuts):
            self._convolution = self._convolution_numpy
        else:
            self._convolution = self._convolution_dot_product

    @staticmethod
    def wake_factor(beam):
        return (-(beam.charge)**2 / (beam.mass * beam.gamma *
                (beam.beta * c)**2) * beam.particlenumber_per_mp)

    def _convolution_dot_product(self, target_times, source_times,
                                 source_moments, source_beta):
        dt = ([target_times] - np.transpose([source_times]))
        wake = self.wake_function(dt, beta=source_beta)
        return np.dot(source_moments, wake)

    def _convolution_numpy(self, target_times, source_times,
                           source_moments, source_beta):
        dt = np.concatenate((target_times - source_times[-1],
                             (target_times - source_times[0])[1:]))
        wake = self.wake_function(dt, beta=source_beta)
        return np.convolve(source_moments, wake, 'valid')

    def signal(self, beam, slice_sets, ages):
        times = [s.convert_to_time(s.z_centers) for s in slice_sets]
        betas = [s.beta for s in slice_sets]
        if self.moment is None:
            moments = [s.n_macroparticles_per_slice for s in slice_sets]
        else:
            moments = [s.n_macroparticles_per_slice *
                       getattr(s, 'mean_' + self.moment) for s in slice_sets]
        n_turns = min(len(ages), self.n_turns_wake)
        acc = 0
        for i in range(n_turns):
            acc += self._convolution(times[0], times[i] + ages[i],
                                     moments[i], betas[i])
        return self.wake_factor(beam) * acc

    def apply(self, beam, slice_sets, ages):
        kick = self.signal(beam, slice_sets, ages)
        ss = slice_sets[0]
        p = ss.particles_within_cuts
        s = ss.slice_index_of_particle[p]
        arr = getattr(beam, self.target)
        if self.quad is None:
            arr[p] += np.take(kick, s)
        else:
            arr[p] += np.take(kick, s) * getattr(beam, self.quad)[p]


def circular_resonator_kicks(slicer, R_shunt, frequency, Q, n_turns_wake=1):
    """CircularResonator (Yokoya X1=Y1=1), wakes.py:402-441, 496-509."""
    wf = resonator_transverse(R_shunt, frequency, Q, 1.)
    return [WakeKick(wf, slicer, n_turns_wake, 'xp', 'x'),
            WakeKick(wf, slicer, n_turns_wake, 'yp', 'y')]


def circular_resistive_wall_kicks(slicer, pipe_radius, length, conductivity,
                                  dt_min, n_turns_wake=1):
    """CircularResistiveWall (Yokoya X1=Y1=1), wakes.py:578-609, 627-640."""
    wf = resistive_wall_transverse(pipe_radius, length, conductivity, dt_min,
                                   1.)
    return [WakeKick(wf, slicer, n_turns_wake, 'xp', 'x'),
            WakeKick(wf, slicer, n_turns_wake, 'yp', 'y')]


def parallel_horizontal_plates_resistive_wall_kicks(slicer, pipe_radius,
                                                    length, conductivity,
                                                    dt_min, n_turns_wake=1):
    """ParallelHorizontalPlatesResistiveWall (wakes.py:643-656): Yokoya
    X1 = pi^2/24, Y1 = pi^2/12, X2 = -pi^2/24, Y2 = pi^2/24, kicks in the
    order of ResistiveWall.get_wake_kicks (wakes.py:577-609): dipole x,
    quadrupole x, dipole y, quadrupole y."""
    def wf(yokoya):
        return resistive_wall_transverse(pipe_radius, length, conductivity,
                                         dt_min, yokoya)
    return [WakeKick(wf(np.pi**2 / 24.), slicer, n_turns_wake, 'xp', 'x'),
            WakeKick(wf(-np.pi**2 / 24.), slicer, n_turns_wake, 'xp', None,
                     quad='x'),
            WakeKick(wf(np.pi**2 / 12.), slicer, n_turns_wake, 'yp', 'y'),
            WakeKick(wf(np.pi**2 / 24.), slicer, n_turns_wake, 'yp', None,
                     quad='y')]


class WakeField(object):
    """WakeField.track, wakes.py:89-145."""

    def __init__(self, slicer, kicks, n_turns_wake_max):
        self.slicer = slicer
        self.kicks = list(kicks)
        self.slice_sets = deque([], maxlen=n_turns_wake_max)
        self.ages = deque([], maxlen=n_turns_wake_max)

    def track(self, beam):
        for i in range(len(self.ages)):
            self.ages[i] += beam.circumference / (beam.beta * c)
        ss = self.slicer.slice(beam, statistics=['mean_x', 'mean_y'])
        self.slice_sets.appendleft(ss)
        self.ages.appendleft(0.)
        for k in self.kicks:
            k.apply(beam, self.slice_sets, self.ages)


# --------------------------------------------------------------------------
# Bunch generation: particles/generators.py, machines/synchrotron.py
# --------------------------------------------------------------------------


def gaussian_bunch(n, seed, gamma, mass, charge, circumference, intensity,
                   epsn_x, epsn_y, beta_x, beta_y, sigma_z, sigma_dp,
                   alpha_x=0., alpha_y=0.):
    """Seeded 6D Gaussian: generators.py:377-395 draw order (x, xp, y, yp,
    z, dp) with gaussian2D (:428-443) and gaussian2D_asymmetrical (:446-459),
    then the linear transverse matcher (:106-153).  The longitudinal plane is
    the unmatched Gaussian with the given sigmas."""
    np.random.seed(seed)
    betagamma = np.sqrt(gamma**2 - 1)
    epsx_geo = epsn_x / betagamma
    epsy_geo = epsn_y / betagamma
    sx = np.sqrt(epsx_geo)
    x = np.random.normal(loc=0., scale=sx, size=n)
    xp = np.random.normal(loc=0., scale=sx, size=n)
    sy = np.sqrt(epsy_geo)
    y = np.random.normal(loc=0., scale=sy, size=n)
    yp = np.random.normal(loc=0., scale=sy, size=n)
    z = np.random.normal(loc=0., scale=sigma_z, size=n)
    dp = np.random.normal(loc=0., scale=sigma_dp, size=n)

    def match(u, up, alpha, beta):
        M00 = np.sqrt(beta)
        M10 = -alpha / np.sqrt(beta)
        M11 = np.sqrt(1. / beta)
        uc = u.copy()
        u = M00 * u + 0 * up
        up = M10 * uc + M11 * up
        return u, up
    x, xp = match(x, xp, alpha_x, beta_x)
    y, yp = match(y, yp, alpha_y, beta_y)
    beam = Beam(dict(x=x, xp=xp, y=y, yp=yp, z=z, dp=dp),
                intensity / n, charge, mass, circumference, gamma)
    return beam
