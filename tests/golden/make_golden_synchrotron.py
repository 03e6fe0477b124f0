"""Generate the Synchrotron fixtures by running the PyHEADTAIL reference.

    python tests/golden/make_golden_synchrotron.py --ref <PyHEADTAIL source tree>

For every entry of cases.SYNCHROTRON_CASES: build the reference's
Synchrotron, draw the seeded bunch with its generate_6D_Gaussian_bunch,
append the extras (a damper after each transverse segment, a resonator
wake at the end) and track with machine.track.  Stored in
synchrotron/<name>.npz: the spec, the one-turn map's element classes,
Q_s, circumference, the initial coordinates and those after the last turn.
"""
import argparse
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import cases as C  # noqa: E402
from make_golden import COORDS, build_reference  # noqa: E402


def run(name, spec):
    from scipy.constants import e, m_p
    from PyHEADTAIL.feedback.transverse_damper import TransverseDamper
    from PyHEADTAIL.general.printers import SilentPrinter
    from PyHEADTAIL.impedances.wakes import CircularResonator, WakeField
    from PyHEADTAIL.machines.synchrotron import Synchrotron
    from PyHEADTAIL.particles.slicing import UniformBinSlicer
    sp = SilentPrinter()
    kw = dict(spec['machine'])
    for k in ('s', 'alpha_x', 'beta_x', 'D_x', 'alpha_y', 'beta_y', 'D_y',
              'accQ_x', 'accQ_y'):
        if isinstance(kw.get(k), list):
            kw[k] = np.array(kw[k])
    machine = Synchrotron(charge=e, mass=m_p, **kw)
    b = spec['bunch']
    np.random.seed(b['seed'])
    bunch = machine.generate_6D_Gaussian_bunch(
        b['n'], b['intensity'], b['epsn_x'], b['epsn_y'], b['sigma_z'])
    rec = {'spec': json.dumps(spec)}
    for k in COORDS:
        rec['init_' + k] = getattr(bunch, k).copy()
    if spec['damper_after_segments']:
        dx, dy = spec['damper_after_segments']
        machine.install_after_each_transverse_segment(
            TransverseDamper(dx, dy, printer=sp))
    if spec['wake']:
        w = spec['wake']
        machine.one_turn_map.append(WakeField(
            UniformBinSlicer(w['n_slices'], z_cuts=tuple(C.Z_CUTS),
                             warningprinter=sp),
            CircularResonator(w['R'], w['f'], w['Q'], printer=sp)))
    rec['elements'] = np.array([type(m).__name__
                                for m in machine.one_turn_map])
    rec['Q_s'] = np.float64(machine.Q_s)
    rec['circumference'] = np.float64(machine.circumference)
    rec['gamma'] = np.float64(machine.gamma)
    for _ in range(spec['n_turns']):
        machine.track(bunch)
    for k in COORDS:
        rec['final_' + k] = getattr(bunch, k).copy()
    os.makedirs(os.path.join(HERE, 'synchrotron'), exist_ok=True)
    np.savez_compressed(os.path.join(HERE, 'synchrotron', name + '.npz'), **rec)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--ref', required=True,
                    help='PyHEADTAIL source tree (read only)')
    ap.add_argument('--scratch', default='/tmp/phk_refbuild')
    ap.add_argument('cases', nargs='*')
    a = ap.parse_args()
    build_reference(a.ref, a.scratch)
    for name in (a.cases or sorted(C.SYNCHROTRON_CASES)):
        run(name, C.SYNCHROTRON_CASES[name])
        print('wrote', name)


if __name__ == '__main__':
    main()
