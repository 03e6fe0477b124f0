"""Golden traces of the reference's broadband-resonator instability test
(tests/simulation_tests/test_bb_resonator.py:11-129 of PyHEADTAIL: smooth
machine at 26 GeV/c, two-harmonic RF (h 4620 and 4 x 4620) in its
non-linear mode, CircularResonator(10.2e6, 1.3e9, 1) on a
UniformBinSlicer(200, n_sigma_z=6), 1e5 macroparticles, 3000 turns; growth
rates 59e-4 (x) and 25e-4 (y) per turn within 5 %), made by running
PyHEADTAIL itself:

    python tests/golden/make_golden_bb_resonator.py --ref <PyHEADTAIL source tree>

The bunch is the reference's RF-bucket-matched Gaussian (numpy seed 3),
rounded to float32 so that the fixture stays small; the reference then
tracks that rounded bunch and the mean_x and mean_y of every turn are
stored with the initial coordinates and the element order in
tests/golden/bb_resonator/.
"""
import argparse
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import make_golden as MG  # noqa: E402

N_PART, NP_SEED, N_TURNS, FIT_FROM = 100000, 3, 3000, 1500
PATH = os.path.join(HERE, 'bb_resonator', 'bb_resonator_1e5.npz')


def machine_parameters():
    """test_bb_resonator.py:18-68."""
    from scipy.constants import c, e
    return dict(intensity=2.5e11, epsn_x=2e-6, epsn_y=2e-6, sigma_z=0.23,
                circumference=6911.5038378975451, p0=26e9 * e / c,
                beta_x=54.644808743169399, beta_y=54.509415262636274,
                Q_x=20.13, Q_y=20.18, alpha=0.0030864197530864196,
                h=[4620, 4 * 4620], V=[4.5e6, 0.45e6], dphi=[0., np.pi],
                R_shunt=10.2e6, frequency=1.3e9, Q=1., n_slices=200,
                n_sigma_z=6)


def growth_rates(x, y, first=FIT_FROM):
    """test_bb_resonator.py:99-118: slope of the log of the Hilbert envelope
    from turn ``first`` on."""
    from scipy.signal import hilbert
    from scipy.stats import linregress
    turns = np.arange(len(x))
    return tuple(linregress(turns[first:], np.log(np.abs(hilbert(u))[first:]))[0]
                 for u in (x, y))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--ref', required=True,
                    help='PyHEADTAIL source tree (read only)')
    ap.add_argument('--scratch', default='/tmp/phk_refbuild')
    a = ap.parse_args()
    MG.build_reference(a.ref, a.scratch)
    MG.patch_reference_numpy2()
    from scipy.constants import e, m_p
    from PyHEADTAIL.impedances import wakes
    from PyHEADTAIL.machines.synchrotron import Synchrotron
    from PyHEADTAIL.particles.slicing import UniformBinSlicer
    p = machine_parameters()
    machine = Synchrotron(
        optics_mode='smooth', circumference=p['circumference'], n_segments=1,
        beta_x=p['beta_x'], beta_y=p['beta_y'], D_x=0.0, D_y=0.0,
        accQ_x=p['Q_x'], accQ_y=p['Q_y'], Qp_x=0.0, Qp_y=0.0,
        alpha_mom_compaction=p['alpha'], longitudinal_mode='non-linear',
        h_RF=p['h'], V_RF=p['V'], dphi_RF=p['dphi'], p_increment=0.,
        p0=p['p0'], charge=e, mass=m_p)
    wake = wakes.CircularResonator(p['R_shunt'], p['frequency'], p['Q'])
    machine.one_turn_map.append(wakes.WakeField(
        UniformBinSlicer(p['n_slices'], n_sigma_z=p['n_sigma_z']), wake))
    np.random.seed(NP_SEED)
    bunch = machine.generate_6D_Gaussian_bunch_matched(
        n_macroparticles=N_PART, intensity=p['intensity'],
        epsn_x=p['epsn_x'], epsn_y=p['epsn_y'], sigma_z=p['sigma_z'])
    init = {}
    for k in ('x', 'xp', 'y', 'yp', 'z', 'dp'):
        init[k] = getattr(bunch, k).astype(np.float32)
        getattr(bunch, k)[:] = init[k].astype(np.float64)
    kinds = [type(m).__name__ for m in machine.one_turn_map]
    x = np.zeros(N_TURNS)
    y = np.zeros(N_TURNS)
    for i in range(N_TURNS):
        for m in machine.one_turn_map:
            m.track(bunch)
        x[i], y[i] = bunch.mean_x(), bunch.mean_y()
    rx, ry = growth_rates(x, y)
    os.makedirs(os.path.dirname(PATH), exist_ok=True)
    np.savez_compressed(PATH, mean_x=x, mean_y=y, growth_rate_x=rx,
                        growth_rate_y=ry, gamma=np.float64(bunch.gamma),
                        elements=np.array(kinds),
                        **{'init_' + k: v for k, v in init.items()})
    print('wrote', PATH, 'growth rates %.4e / %.4e per turn' % (rx, ry),
          kinds)


if __name__ == '__main__':
    main()
