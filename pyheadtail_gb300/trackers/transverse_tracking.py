"""Transverse linear segment maps for the GPU turn loop.

Mirrors PyHEADTAIL's trackers/transverse_tracking.py:
``TransverseSegmentMap`` (:17-196) and ``TransverseMap`` (:199-358), same
constructors, same I / J matrices (:71-103), same dispersion switch (:65-69)
and the same phase advance ``(dQ + detuning) * 2 pi``.  ``track(beam)``
appends a transverse op to the beam's pending program; without detuners the
matrix entries are host scalars computed exactly as the reference does,
with detuners the per-particle phase advance, its sine / cosine and the
matrix are evaluated in the fused kernel.
"""
import numpy as np

from .. import _engine as E
from .. import _native as N
from ..general.element import Element, Printing
from .detuners import AmplitudeDetuningSegment, ChromaticitySegment


class TransverseSegmentMap(Element):
    """Linear transport of (x, xp, y, yp) over one ring segment."""

    def __init__(self, alpha_x_s0, beta_x_s0, D_x_s0, alpha_x_s1, beta_x_s1,
                 D_x_s1, alpha_y_s0, beta_y_s0, D_y_s0, alpha_y_s1, beta_y_s1,
                 D_y_s1, dQ_x, dQ_y, *args, **kwargs):
        self.D_x_s0, self.D_x_s1 = D_x_s0, D_x_s1
        self.D_y_s0, self.D_y_s1 = D_y_s0, D_y_s1
        self.dQ_x, self.dQ_y = dQ_x, dQ_y
        self._build_segment_map(alpha_x_s0, beta_x_s0, alpha_x_s1, beta_x_s1,
                                alpha_y_s0, beta_y_s0, alpha_y_s1, beta_y_s1)
        self.segment_detuners = kwargs.pop('segment_detuners', [])
        for d in self.segment_detuners:
            if not isinstance(d, (ChromaticitySegment,
                                  AmplitudeDetuningSegment)):
                raise TypeError('the GPU transverse map fuses chromaticity and '
                                'amplitude detuning only, got %r' % (d,))
        self.with_dispersion = not np.allclose(
            [D_x_s0, D_x_s1, D_y_s0, D_y_s1], np.zeros(4), atol=1e-3)

    def _build_segment_map(self, alpha_x_s0, beta_x_s0, alpha_x_s1, beta_x_s1,
                           alpha_y_s0, beta_y_s0, alpha_y_s1, beta_y_s1):
        """transverse_tracking.py:71-103."""
        I = np.zeros((4, 4))
        J = np.zeros((4, 4))
        I[0, 0] = np.sqrt(beta_x_s1 / beta_x_s0)
        I[0, 1] = 0.
        I[1, 0] = (np.sqrt(1. / (beta_x_s0 * beta_x_s1)) *
                   (alpha_x_s0 - alpha_x_s1))
        I[1, 1] = np.sqrt(beta_x_s0 / beta_x_s1)
        I[2, 2] = np.sqrt(beta_y_s1 / beta_y_s0)
        I[2, 3] = 0.
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
        self.I, self.J = I, J

    _ENTRIES = ((0, 0), (0, 1), (1, 0), (1, 1), (2, 2), (2, 3), (3, 2), (3, 3))

    def _op(self, beam):
        flags = N.FLAG_DISPERSION if self.with_dispersion else 0
        D = (self.D_x_s0, self.D_x_s1, self.D_y_s0, self.D_y_s1)
        p = {16 + i: float(v) for i, v in enumerate(D)}
        pf = {32 + i: np.float32(v) for i, v in enumerate(D)}
        I, J = self.I, self.J
        if not self.segment_detuners:
            # transverse_tracking.py:150-193 with scalar phase advance
            dphi_x = self.dQ_x * (2. * np.pi)
            dphi_y = self.dQ_y * (2. * np.pi)
            c_x, c_y = np.cos(dphi_x), np.cos(dphi_y)
            s_x, s_y = np.sin(dphi_x), np.sin(dphi_y)
            for i, (a, b) in enumerate(self._ENTRIES):
                cc, ss = (c_x, s_x) if a < 2 else (c_y, s_y)
                m = I[a, b] * cc + J[a, b] * ss
                p[i] = float(m)
                # precision form: float-float entries, so that the FP32 map
                # carries no systematic rounding of its matrix
                pf[i], pf[40 + i] = E.split_ff(m)
            return E.Op(N.OP_TRANSVERSE, flags, p, pf)
        flags |= N.FLAG_DETUNED
        mask = 0
        for i, (a, b) in enumerate(self._ENTRIES):
            p[i] = float(I[a, b])
            p[8 + i] = float(J[a, b])
            pf[i], pf[40 + i] = E.split_ff(I[a, b])
            pf[8 + i], pf[48 + i] = E.split_ff(J[a, b])
            mask |= (I[a, b] != 0) << i
            mask |= (J[a, b] != 0) << (8 + i)
        p[20], p[21], p[22] = float(self.dQ_x), float(self.dQ_y), 2. * np.pi
        # base of the angle-addition sin/cos: the undetuned phase advance,
        # rounded exactly as the reference rounds dQ * 2 pi, and its sin/cos
        for k, q in ((23, self.dQ_x), (26, self.dQ_y)):
            phi0 = q * (2. * np.pi)
            p[k], p[k + 1], p[k + 2] = (float(phi0), float(np.sin(phi0)),
                                        float(np.cos(phi0)))
        # precision form: phase in turns, integer part removed exactly
        for k, q in ((16, self.dQ_x), (18, self.dQ_y)):
            frac = float(q) - np.floor(float(q))
            pf[k], pf[k + 1] = E.split_ff(frac)
        dets = [d._pack(beam) for d in self.segment_detuners]
        return E.Op(N.OP_TRANSVERSE, flags, p, pf, dets, ij_mask=mask)

    def track(self, beam):
        beam._engine.enqueue(self._op(beam))


class TransverseMap(Printing):
    """One-turn transverse map split into segments at the positions s
    (transverse_tracking.py:199-358)."""

    def __init__(self, s, alpha_x, beta_x, D_x, alpha_y, beta_y, D_y,
                 accQ_x, accQ_y, detuners=[], *args, **kwargs):
        self.s = s
        self.alpha_x, self.beta_x, self.D_x = alpha_x, beta_x, D_x
        self.alpha_y, self.beta_y, self.D_y = alpha_y, beta_y, D_y
        self.accQ_x, self.accQ_y = accQ_x, accQ_y
        self.detuner_collections = detuners
        self.segment_maps = []
        self._generate_segment_maps()
        if any(self.D_x) or any(self.D_y):
            self.prints('Non-zero dispersion in tracking: ensure the beam has '
                        'been generated being matched to the correct '
                        'dispersion!')

    def _generate_segment_maps(self):
        """transverse_tracking.py:275-329."""
        segment_length = np.diff(self.s) / self.s[-1]
        dQ_x = (self.accQ_x * segment_length if np.ndim(self.accQ_x) == 0
                else np.diff(self.accQ_x))
        dQ_y = (self.accQ_y * segment_length if np.ndim(self.accQ_y) == 0
                else np.diff(self.accQ_y))
        n_segments = len(self.s) - 1
        dmu_x = dQ_x / np.atleast_1d(self.accQ_x)[-1]
        dmu_y = dQ_y / np.atleast_1d(self.accQ_y)[-1]
        for seg in range(n_segments):
            s0 = seg % n_segments
            s1 = (seg + 1) % n_segments
            for detuner in self.detuner_collections:
                detuner.generate_segment_detuner(
                    dmu_x[s0], dmu_y[s0],
                    alpha_x=self.alpha_x[s0], beta_x=self.beta_x[s0],
                    alpha_y=self.alpha_y[s0], beta_y=self.beta_y[s0])
            self.segment_maps.append(TransverseSegmentMap(
                self.alpha_x[s0], self.beta_x[s0], self.D_x[s0],
                self.alpha_x[s1], self.beta_x[s1], self.D_x[s1],
                self.alpha_y[s0], self.beta_y[s0], self.D_y[s0],
                self.alpha_y[s1], self.beta_y[s1], self.D_y[s1],
                dQ_x[seg], dQ_y[seg],
                segment_detuners=[d[seg] for d in self.detuner_collections]))

    def get_injection_optics(self, for_particle_generation=False):
        disp = 'dispersion' if for_particle_generation else 'D'
        return {'alpha_x': self.alpha_x[0], 'beta_x': self.beta_x[0],
                disp + '_x': self.D_x[0], 'alpha_y': self.alpha_y[0],
                'beta_y': self.beta_y[0], disp + '_y': self.D_y[0]}

    def __len__(self):
        return len(self.segment_maps)

    def __getitem__(self, key):
        return self.segment_maps[key]
