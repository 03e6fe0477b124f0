"""The oracle on the reference's broadband-resonator instability test
(tests/simulation_tests/test_bb_resonator.py:11-129 of PyHEADTAIL), from
the fixture made by tests/golden/make_golden_bb_resonator.py with
PyHEADTAIL itself: the RF-bucket-matched 1e5-particle bunch (rounded to
float32), the machine's element order [RFSystems, TransverseSegmentMap,
WakeField], two-harmonic RF in the non-linear mode, CircularResonator
(10.2e6, 1.3e9, 1) on UniformBinSlicer(200, n_sigma_z=6) -- cuts that
follow the bunch every turn.  Over 3000 turns of a growing instability
the oracle's centroids must equal the reference's to 1e-9 of their largest
value, its growth rates (fitted as the reference test fits them) must
equal the reference's to 1e-6 relative, and both must meet the reference
test's own bars (59e-4 and 25e-4 per turn within 5 %)."""
import os
import sys

import numpy as np
import pytest
from scipy.constants import c, e, m_p

from oracle import turn_loop as T

GOLDEN = os.path.join(os.path.dirname(__file__), 'golden')
sys.path.insert(0, GOLDEN)


def _elements(p, gamma):
    C = p['circumference']
    z2 = np.zeros(2)
    bx = np.array([p['beta_x'], p['beta_x']])
    by = np.array([p['beta_y'], p['beta_y']])
    rf = T.RFSystems(C, p['h'], p['V'], p['dphi'], [p['alpha']], gamma,
                     charge=e, mass=m_p)
    # Q' = 0: the reference's Synchrotron adds no detuner
    segs = T.transverse_map([0., C], z2, bx, z2, z2, by, z2, p['Q_x'],
                            p['Q_y'], chroma=None, amplitude=None)
    sl = T.UniformBinSlicer(p['n_slices'], z_cuts=None,
                            n_sigma_z=p['n_sigma_z'])
    kicks = T.circular_resonator_kicks(sl, p['R_shunt'], p['frequency'],
                                       p['Q'])
    return [rf] + list(segs) + [T.WakeField(sl, kicks, 1)]


@pytest.mark.timeout(900)
def test_oracle_reproduces_reference_bb_resonator_growth():
    import make_golden_bb_resonator as G
    p = G.machine_parameters()
    with np.load(G.PATH) as f:
        g = {k: f[k] for k in f.files}
    assert list(g['elements']) == ['RFSystems', 'TransverseSegmentMap',
                                   'WakeField']
    coords = {k: g['init_' + k].astype(np.float64)
              for k in ('x', 'xp', 'y', 'yp', 'z', 'dp')}
    # Synchrotron's gamma follows from its p0 (synchrotron.py)
    gamma = np.sqrt(1 + (p['p0'] / (m_p * c))**2)
    assert gamma == float(g['gamma'])
    beam = T.Beam(coords, p['intensity'] / len(coords['x']), e, m_p,
                  p['circumference'], gamma)
    els = _elements(p, gamma)
    x = np.zeros(G.N_TURNS)
    y = np.zeros(G.N_TURNS)
    for i in range(G.N_TURNS):
        for m in els:
            m.track(beam)
        x[i], y[i] = beam.mean_x(), beam.mean_y()
    for got, ref in ((x, g['mean_x']), (y, g['mean_y'])):
        scale = np.max(np.abs(ref))
        assert np.max(np.abs(got - ref)) <= 1e-9 * scale, \
            np.max(np.abs(got - ref)) / scale
    rx, ry = G.growth_rates(x, y)
    assert abs(rx - float(g['growth_rate_x'])) <= 1e-6 * abs(rx)
    assert abs(ry - float(g['growth_rate_y'])) <= 1e-6 * abs(ry)
    # the reference test's bars
    assert np.isclose(rx, 59e-4, rtol=5e-2), rx
    assert np.isclose(ry, 25e-4, rtol=5e-2), ry
