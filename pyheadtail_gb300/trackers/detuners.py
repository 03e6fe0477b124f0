"""Incoherent detuning (chromaticity, amplitude detuning) for the GPU
transverse map.

Mirrors PyHEADTAIL's trackers/detuners.py: ``SegmentDetuner`` (:34-45),
``ChromaticitySegment`` (:48-98), ``AmplitudeDetuningSegment`` (:101-151),
``DetunerCollection`` (:154-198), ``AmplitudeDetuning`` (:201-281) and
``Chromaticity`` (:283-312), with the same constructor arguments and
segment generation.  The per-particle detuning is evaluated inside the fused
track kernel: each segment detuner describes itself to the kernel through
``_pack(beam)``.  ``detune(beam)`` stays available and returns device
tensors (it is not used by the hot path).
"""
from abc import ABCMeta, abstractmethod
from math import factorial

import numpy as np
from scipy.constants import c, e

from .. import _engine as E
from .. import _native as N


class SegmentDetuner(object, metaclass=ABCMeta):

    @abstractmethod
    def detune(self, beam):
        pass


class ChromaticitySegment(SegmentDetuner):
    """dQ = sum_i Qp_i / (i+1)! * dp^(i+1) (detuners.py:48-98)."""

    def __init__(self, dQp_x, dQp_y):
        dQp_x = np.atleast_1d(dQp_x)
        dQp_y = np.atleast_1d(dQp_y)
        self.coeffs_x = [q / float(factorial(i + 1)) for i, q in enumerate(dQp_x)]
        self.coeffs_y = [q / float(factorial(i + 1)) for i, q in enumerate(dQp_y)]
        if len(self.coeffs_x) > N.PHK_MAX_POLY or \
                len(self.coeffs_y) > N.PHK_MAX_POLY:
            raise ValueError('chromaticity orders above %d are not supported'
                             % N.PHK_MAX_POLY)
        # the reference's polyval path (order > 3) prepends one zero
        # coefficient per call (detuners.py:95-97): count the calls per
        # plane; the kernel and calc_detuning_x / _y read the same counts
        self._calls = [0, 0]
        self.calc_detuning_x = self._plane_detuning(0)
        self.calc_detuning_y = self._plane_detuning(1)

    def _coeffs(self, q):
        return self.coeffs_x if q == 0 else self.coeffs_y

    def _bump(self, q):
        if len(self._coeffs(q)) > 3:
            self._calls[q] += 1

    def _extra_of(self, q):
        return max(self._calls[q] - 1, 0) if len(self._coeffs(q)) > 3 else 0

    def _plane_detuning(self, q):
        def calc_detuning(dp):
            """The plane's detuning of an array dp (numpy or torch):
            ChromaticitySegment.calc_detuning_x / _y (detuners.py:74-98)."""
            self._bump(q)
            return _chroma_poly(self._coeffs(q), self._extra_of(q), dp)
        return calc_detuning

    @staticmethod
    def _make_calc_detuning(Qp):
        """A stand-alone detuning polynomial of the chromaticities Qp
        (detuners.py:74-98): orders 1-3 written out, higher orders with
        the reference's zero prepended on every call."""
        coeffs = [Qp[i] / float(factorial(i + 1)) for i in range(len(Qp))]
        calls = [0]

        def calc_detuning(dp):
            extra = 0
            if len(coeffs) > 3:
                calls[0] += 1
                extra = calls[0] - 1
            return _chroma_poly(coeffs, extra, dp)
        return calc_detuning

    def _pack(self, beam):
        self._bump(0)
        self._bump(1)
        c = {}
        cf = {}
        for i, v in enumerate(self.coeffs_x):
            c[i] = float(v)
            cf[i] = np.float32(v)
        for i, v in enumerate(self.coeffs_y):
            c[8 + i] = float(v)
            cf[8 + i] = np.float32(v)
        return E.DetunerPack(N.DET_CHROMA, c, cf, nx=len(self.coeffs_x),
                             ny=len(self.coeffs_y),
                             zx=self._extra_of(0), zy=self._extra_of(1))

    def detune(self, beam):
        """detuners.py:64-69 (device tensors; the fused kernel evaluates
        the same polynomials in the track pass)."""
        dp = beam.dp.double()
        return self.calc_detuning_x(dp), self.calc_detuning_y(dp)


def _chroma_poly(coeffs, extra, dp):
    """(c0 + (c1 + ...) dp) dp times dp**extra: the reference's explicit
    orders 1-3 and, above, np.polynomial.polynomial.polyval over the
    coefficients with 1 + extra zeros prepended (Horner: the zeros only
    multiply by dp, exactly)."""
    if len(coeffs) == 1:
        r = coeffs[0] * dp
    else:
        r = coeffs[-1] + 0 * dp
        for cc in coeffs[-2::-1]:
            r = cc + r * dp
        r = r * dp
    for _ in range(extra):
        r = r * dp
    return r


class AmplitudeDetuningSegment(SegmentDetuner):
    """Linear amplitude detuning (detuners.py:101-151); the normalisation
    to beam.p0 is done when the segment is tracked."""

    def __init__(self, dapp_x, dapp_y, dapp_xy, dapp_yx, alpha_x, beta_x,
                 alpha_y, beta_y):
        self.alpha_x, self.beta_x = alpha_x, beta_x
        self.alpha_y, self.beta_y = alpha_y, beta_y
        self.dapp_x, self.dapp_y = dapp_x, dapp_y
        self.dapp_xy, self.dapp_yx = dapp_xy, dapp_yx

    def _pack(self, beam):
        ax, bx, ay, by = self.alpha_x, self.beta_x, self.alpha_y, self.beta_y
        c1x = (1 + ax**2) / bx
        c1y = (1 + ay**2) / by
        p0 = beam.p0
        vals = [self.dapp_x, self.dapp_y, self.dapp_xy, self.dapp_yx,
                c1x, 2 * ax, bx, c1y, 2 * ay, by, p0, 1. / p0]
        c = {i: float(v) for i, v in enumerate(vals)}
        cf = {0: np.float32(self.dapp_x / p0), 1: np.float32(self.dapp_y / p0),
              2: np.float32(self.dapp_xy / p0),
              3: np.float32(self.dapp_yx / p0),
              4: np.float32(c1x), 5: np.float32(2 * ax), 6: np.float32(bx),
              7: np.float32(c1y), 8: np.float32(2 * ay), 9: np.float32(by)}
        return E.DetunerPack(N.DET_AMPLITUDE, c, cf)

    def detune(self, beam):
        x, xp = beam.x.double(), beam.xp.double()
        y, yp = beam.y.double(), beam.yp.double()
        Jx = 1 / 2 * ((1 + self.alpha_x**2) / self.beta_x * x**2 +
                      2 * self.alpha_x * x * xp + self.beta_x * xp**2)
        Jy = 1 / 2 * ((1 + self.alpha_y**2) / self.beta_y * y**2 +
                      2 * self.alpha_y * y * yp + self.beta_y * yp**2)
        dQ_x = (self.dapp_x * Jx + self.dapp_xy * Jy) / beam.p0
        dQ_y = (self.dapp_y * Jy + self.dapp_yx * Jx) / beam.p0
        return dQ_x, dQ_y


class DetunerCollection(object, metaclass=ABCMeta):

    @abstractmethod
    def generate_segment_detuner(self, dmu_x, dmu_y, **kwargs):
        pass

    def __len__(self):
        return len(self.segment_detuners)

    def __getitem__(self, key):
        return self.segment_detuners[key]


class AmplitudeDetuning(DetunerCollection):
    """One-turn amplitude detuning app_x, app_y, app_xy (detuners.py:201-281),
    not normalised to p0."""

    def __init__(self, app_x, app_y, app_xy):
        self.app_x = app_x
        self.app_y = app_y
        self.app_xy = app_xy
        self.segment_detuners = []

    @classmethod
    def from_octupole_currents_LHC(cls, i_focusing, i_defocusing):
        """LHC Landau octupole detuning (detuners.py:222-264)."""
        i_max = 550.
        E_max = 7000.
        app_x = E_max * (267065. * i_focusing / i_max -
                         7856. * i_defocusing / i_max)
        app_y = E_max * (9789. * i_focusing / i_max -
                         277203. * i_defocusing / i_max)
        app_xy = E_max * (-102261. * i_focusing / i_max +
                          93331. * i_defocusing / i_max)
        convert_to_SI = e / (1.e-9 * c)
        return cls(app_x * convert_to_SI, app_y * convert_to_SI,
                   app_xy * convert_to_SI)

    def generate_segment_detuner(self, dmu_x, dmu_y, **kwargs):
        detuner = AmplitudeDetuningSegment(
            self.app_x * dmu_x, self.app_y * dmu_y, self.app_xy * dmu_x,
            self.app_xy * dmu_y, **kwargs)
        self.segment_detuners.append(detuner)


class Chromaticity(DetunerCollection):
    """One-turn chromaticities Q'_x, Q''_x, ... (detuners.py:283-312)."""

    def __init__(self, Qp_x, Qp_y):
        self.Qp_x = np.atleast_1d(Qp_x)
        self.Qp_y = np.atleast_1d(Qp_y)
        self.segment_detuners = []

    def generate_segment_detuner(self, dmu_x, dmu_y, **kwargs):
        dQp_x = [Qp * dmu_x for Qp in self.Qp_x]
        dQp_y = [Qp * dmu_y for Qp in self.Qp_y]
        self.segment_detuners.append(ChromaticitySegment(dQp_x, dQp_y))
