"""The oracle on the reference's resistive-wall instability test
(tests/simulation_tests/test_resistive_wall.py:11-120 of PyHEADTAIL), from
the fixture made by tests/golden/make_golden_reswall.py with PyHEADTAIL
itself: the RF-bucket-matched 5e4-particle bunch (rounded to float32), the
machine's element order [RFSystems, TransverseSegmentMap, WakeField], the
parallel horizontal plates resistive wall and UniformChargeSlicer(500,
n_sigma_z=3) with the reference's random remainder draws (Python random,
seed 7).  The oracle's vertical centroid over 1000 turns must equal the
reference's to 1e-9 of its largest value (measured 2e-17 absolute on the
x86 host that made the fixture, the centroid's summation order; the bar
leaves room for another platform's libm over 1000 unstable turns), and the growth rate fitted as the reference
test fits it must meet its bar (70e-4 per turn within 5 %; the fixture's
bunch gives 7.23e-3)."""
import os
import random
import sys

import numpy as np
import pytest
from scipy.constants import c, e, m_p
from scipy.signal import hilbert
from scipy.stats import linregress

from oracle import turn_loop as T

GOLDEN = os.path.join(os.path.dirname(__file__), 'golden')
sys.path.insert(0, GOLDEN)


def _elements(p, gamma):
    C = p['circumference']
    z2 = np.zeros(2)
    b2 = np.array([p['beta'], p['beta']])
    rf = T.RFSystems(C, [p['h']], [p['V']], [p['dphi']], [p['alpha']], gamma,
                     charge=e, mass=m_p)
    segs = T.transverse_map([0., C], z2, b2, z2, z2, b2, z2, p['Q_x'], p['Q_y'],
                            chroma=(p['Q_x'] * p['xi'], p['Q_y'] * p['xi']),
                            amplitude=None)
    sl = T.UniformChargeSlicer(p['n_slices'], n_sigma_z=p['n_sigma_z'])
    kicks = T.parallel_horizontal_plates_resistive_wall_kicks(
        sl, p['pipe_radius'], p['length'], p['conductivity'], p['dt_min'])
    return [rf] + list(segs) + [T.WakeField(sl, kicks, 1)]


@pytest.mark.timeout(900)
def test_oracle_reproduces_reference_resistive_wall_growth():
    import make_golden_reswall as G
    p = G.machine_parameters()
    with np.load(os.path.join(GOLDEN, 'reswall', 'reswall_5e4.npz')) as f:
        g = {k: f[k] for k in f.files}
    assert list(g['elements']) == ['RFSystems', 'TransverseSegmentMap',
                                   'WakeField']
    coords = {k: g['init_' + k].astype(np.float64)
              for k in ('x', 'xp', 'y', 'yp', 'z', 'dp')}
    # Synchrotron's gamma follows from its p0 (synchrotron.py)
    gamma = np.sqrt(1 + (p['p0'] / (m_p * c))**2)
    beam = T.Beam(coords, p['intensity'] / len(coords['x']), e, m_p,
                  p['circumference'], gamma)
    els = _elements(p, gamma)
    random.seed(G.PY_SEED)
    y = np.zeros(G.N_TURNS)
    for i in range(G.N_TURNS):
        for m in els:
            m.track(beam)
        y[i] = beam.mean_y()
    ref = g['mean_y']
    scale = np.max(np.abs(ref))
    assert np.max(np.abs(y - ref)) <= 1e-9 * scale, np.max(np.abs(y - ref))
    ampl = np.abs(hilbert(y))
    rate = linregress(np.arange(G.N_TURNS)[100:], np.log(ampl[100:]))[0]
    assert abs(rate - float(g['growth_rate'])) <= 1e-6 * abs(rate)
    assert np.isclose(rate, 70e-4, rtol=5e-2), rate
