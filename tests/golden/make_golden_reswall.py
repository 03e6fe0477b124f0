"""Golden trace of the reference's resistive-wall instability test
(tests/simulation_tests/test_resistive_wall.py:11-120 of PyHEADTAIL: smooth
machine, RF h=7 in its non-linear mode, parallel horizontal plates resistive
wall, UniformChargeSlicer(500, n_sigma_z=3), 1000 turns, vertical growth
rate 70e-4 per turn within 5 %), made by running PyHEADTAIL itself:

    python tests/golden/make_golden_reswall.py --ref <PyHEADTAIL source tree>

The bunch is the reference's RF-bucket-matched Gaussian (5e4 particles,
numpy seed 2), rounded to float32 so that the fixture stays small; the
reference then tracks that rounded bunch (Python's random seeded with 7
for the uniform-charge slicer's remainder draws) and the mean_y of every
turn is stored with the initial coordinates in tests/golden/reswall/.
"""
import argparse
import os
import random
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import make_golden as MG  # noqa: E402

N_PART, NP_SEED, PY_SEED, N_TURNS = 50000, 2, 7, 1000


def machine_parameters():
    from scipy.constants import c, e, m_p
    E_kin = 1.4e9
    gamma = 1 + E_kin / (m_p * c**2 / e)
    return dict(circumference=2 * np.pi * 100, gamma=gamma,
                p0=np.sqrt(gamma**2 - 1) * m_p * c, beta=16., Q_x=6.22,
                Q_y=6.25, xi=-0.1, alpha=0.027, h=7, V=20e3, dphi=np.pi,
                intensity=1.6e12, epsn=2e-6, sigma_z=12.4, n_slices=500,
                n_sigma_z=3, conductivity=1e6, pipe_radius=0.0356,
                length=10000., dt_min=1e-12)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--ref', required=True,
                    help='PyHEADTAIL source tree (read only)')
    ap.add_argument('--scratch', default='/tmp/pyht_ref')
    a = ap.parse_args()
    MG.build_reference(a.ref, a.scratch)
    MG.patch_reference_numpy2()
    from scipy.constants import e, m_p
    from scipy.signal import hilbert
    from scipy.stats import linregress
    from PyHEADTAIL.impedances import wakes
    from PyHEADTAIL.machines.synchrotron import Synchrotron
    from PyHEADTAIL.particles.slicing import UniformChargeSlicer
    p = machine_parameters()
    machine = Synchrotron(
        optics_mode='smooth', circumference=p['circumference'], n_segments=1,
        beta_x=p['beta'], beta_y=p['beta'], D_x=0.0, D_y=0.0,
        accQ_x=p['Q_x'], accQ_y=p['Q_y'], Qp_x=p['Q_x'] * p['xi'],
        Qp_y=p['Q_y'] * p['xi'], alpha_mom_compaction=p['alpha'],
        longitudinal_mode='non-linear', h_RF=p['h'], V_RF=p['V'],
        dphi_RF=p['dphi'], p_increment=0.0, p0=p['p0'], charge=e, mass=m_p)
    wake = wakes.ParallelHorizontalPlatesResistiveWall(
        conductivity=p['conductivity'], pipe_radius=p['pipe_radius'],
        resistive_wall_length=p['length'], dt_min=p['dt_min'])
    machine.one_turn_map.append(wakes.WakeField(
        UniformChargeSlicer(p['n_slices'], n_sigma_z=p['n_sigma_z']), wake))
    np.random.seed(NP_SEED)
    bunch = machine.generate_6D_Gaussian_bunch_matched(
        n_macroparticles=N_PART, intensity=p['intensity'], epsn_x=p['epsn'],
        epsn_y=p['epsn'], sigma_z=p['sigma_z'])
    init = {}
    for k in ('x', 'xp', 'y', 'yp', 'z', 'dp'):
        init[k] = getattr(bunch, k).astype(np.float32)
        getattr(bunch, k)[:] = init[k].astype(np.float64)
    kinds = [type(m).__name__ for m in machine.one_turn_map]
    random.seed(PY_SEED)
    y = np.zeros(N_TURNS)
    for i in range(N_TURNS):
        for m in machine.one_turn_map:
            m.track(bunch)
        y[i] = bunch.mean_y()
    ampl = np.abs(hilbert(y))
    rate = linregress(np.arange(N_TURNS)[100:], np.log(ampl[100:]))[0]
    path = os.path.join(HERE, 'reswall', 'reswall_5e4.npz')
    np.savez_compressed(path, mean_y=y, growth_rate=rate,
                        elements=np.array(kinds),
                        **{'init_' + k: v for k, v in init.items()})
    print('wrote', path, 'growth rate %.4e per turn' % rate, kinds)


if __name__ == '__main__':
    main()
