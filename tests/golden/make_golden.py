"""Generate the golden fixtures by running the PyHEADTAIL reference itself.

Run in a container where the reference source tree is present (it is read
only, so it is copied and its one Cython extension is built in a scratch
directory first):

    python tests/golden/make_golden.py --ref <PyHEADTAIL source tree>

For every case in ``cases.py`` the script draws the seeded bunch with the
reference's own generator (``ParticleGenerator`` + ``gaussian2D`` /
``gaussian2D_asymmetrical``), tracks it through the reference elements and
stores the initial coordinates, the coordinates after the first and the
last turn, the beam scalars and every recorded SliceSet in
``<case>.npz``.  The fixtures are the pinned answers for the oracle
(``tests/test_oracle_golden.py``) and, through the oracle, for the GPU path.
"""
import argparse
import json
import os
import shutil
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import cases as C  # noqa: E402


def build_reference(ref, scratch):
    if not os.path.exists(os.path.join(scratch, 'PyHEADTAIL')):
        shutil.copytree(ref, scratch)
    so = [f for f in os.listdir(os.path.join(scratch, 'PyHEADTAIL',
                                             'cobra_functions'))
          if f.startswith('stats') and f.endswith('.so')]
    if not so:
        subprocess.check_call([sys.executable, 'setup.py', 'build_ext',
                               '--inplace'], cwd=scratch,
                              stdout=subprocess.DEVNULL)
    sys.path.insert(0, scratch)


def patch_reference_numpy2():
    """PyHEADTAIL v1.16.5's UniformChargeSlicer computes its per-slice
    counts as (numpy int64 scalar) * (int32 array), which NumPy 2 promotes
    to int64 (NEP 50); its Cython statistics then reject the buffer
    ("expected 'int' but got 'long'").  Cast the counts back to the int32
    the code intends; every value is unchanged."""
    from PyHEADTAIL.particles import slicing
    orig = slicing.UniformChargeSlicer.compute_sliceset_kwargs
    if getattr(orig, '_int32_counts', False):
        return

    def compute_sliceset_kwargs(self, beam):
        kw = orig(self, beam)
        kw['n_macroparticles_per_slice'] = np.asarray(
            kw['n_macroparticles_per_slice'], dtype=np.int32)
        return kw
    compute_sliceset_kwargs._int32_counts = True
    slicing.UniformChargeSlicer.compute_sliceset_kwargs = compute_sliceset_kwargs


def make_beam(bp):
    from scipy.constants import m_p, e
    from PyHEADTAIL.particles import generators
    gamma = bp['gamma']
    betagamma = np.sqrt(gamma**2 - 1)
    np.random.seed(bp['seed'])
    return generators.ParticleGenerator(
        macroparticlenumber=bp['n'], intensity=bp['intensity'], charge=e,
        mass=m_p, circumference=bp['circumference'], gamma=gamma,
        distribution_x=generators.gaussian2D(bp['epsn_x'] / betagamma),
        alpha_x=bp['alpha_x'], beta_x=bp['beta_x'], D_x=None,
        distribution_y=generators.gaussian2D(bp['epsn_y'] / betagamma),
        alpha_y=bp['alpha_y'], beta_y=bp['beta_y'], D_y=None,
        distribution_z=generators.gaussian2D_asymmetrical(
            bp['sigma_z'], bp['sigma_dp'])).generate()


def make_slicer(sp):
    from PyHEADTAIL.particles.slicing import (UniformBinSlicer,
                                              UniformChargeSlicer)
    from PyHEADTAIL.general.printers import SilentPrinter
    z_cuts = None if sp['z_cuts'] is None else tuple(sp['z_cuts'])
    if sp.get('mode') == 'uniform_charge':
        return UniformChargeSlicer(sp['n_slices'], n_sigma_z=sp['n_sigma_z'],
                                   z_cuts=z_cuts,
                                   warningprinter=SilentPrinter())
    return UniformBinSlicer(sp['n_slices'], n_sigma_z=sp['n_sigma_z'],
                            z_cuts=z_cuts, warningprinter=SilentPrinter())


def make_source(src):
    from PyHEADTAIL.impedances import wakes
    from PyHEADTAIL.general.printers import SilentPrinter
    sp = SilentPrinter()
    if src['type'] == 'resonator':
        args = (src['R'], src['f'], src['Q'])
        kind = src['kind']
        if kind == 'circular':
            return wakes.CircularResonator(*args, n_turns_wake=src['n_turns_wake'],
                                           printer=sp, warningprinter=sp)
        if kind == 'parallel_horizontal':
            return wakes.ParallelHorizontalPlatesResonator(
                *args, n_turns_wake=src['n_turns_wake'], printer=sp,
                warningprinter=sp)
        if kind == 'longitudinal':
            return wakes.Resonator(*args, Yokoya_X1=0, Yokoya_Y1=0,
                                   Yokoya_X2=0, Yokoya_Y2=0, switch_Z=True,
                                   n_turns_wake=src['n_turns_wake'],
                                   printer=sp, warningprinter=sp)
    if src['type'] == 'wake_table':
        return wakes.WakeTable(os.path.join(HERE, src['file']), src['columns'],
                               n_turns_wake=src['n_turns_wake'], printer=sp,
                               warningprinter=sp)
    if src['type'] == 'resistive_wall' and src['kind'] == 'circular':
        return wakes.CircularResistiveWall(
            src['b'], src['L'], src['sigma'], src['dt_min'],
            n_turns_wake=src['n_turns_wake'], printer=sp, warningprinter=sp)
    raise ValueError(src)


def make_elements(spec, beam):
    from scipy.constants import m_p, e
    from PyHEADTAIL.trackers.transverse_tracking import TransverseMap
    from PyHEADTAIL.trackers.detuners import Chromaticity, AmplitudeDetuning
    from PyHEADTAIL.trackers.longitudinal_tracking import RFSystems, LinearMap
    from PyHEADTAIL.impedances.wakes import WakeField
    from PyHEADTAIL.general.printers import SilentPrinter
    sp = SilentPrinter()
    out = []
    for el in spec['elements']:
        t = el['type']
        if t == 'transverse':
            dets = []
            if el['chroma'] is not None:
                dets.append(Chromaticity(*el['chroma']))
            if el['amplitude'] is not None:
                dets.append(AmplitudeDetuning(*el['amplitude']))
            tm = TransverseMap(np.array(el['s']), np.array(el['alpha_x']),
                               np.array(el['beta_x']), np.array(el['D_x']),
                               np.array(el['alpha_y']), np.array(el['beta_y']),
                               np.array(el['D_y']),
                               np.array(el['accQ_x']) if isinstance(
                                   el['accQ_x'], list) else el['accQ_x'],
                               np.array(el['accQ_y']) if isinstance(
                                   el['accQ_y'], list) else el['accQ_y'],
                               dets, printer=sp)
            out.extend(('map', m) for m in tm)
        elif t == 'rf':
            out.append(('map', RFSystems(
                beam.circumference, el['h'], el['V'], el['dphi'], el['alpha'],
                beam.gamma, p_increment=el['p_increment'], D_x=el['D_x'],
                D_y=el['D_y'], shrink_transverse=el['shrink_transverse'],
                charge=e, mass=m_p, printer=sp, warningprinter=sp)))
        elif t == 'linear_map':
            out.append(('map', LinearMap(el['alpha'], beam.circumference,
                                         el['Q_s'], D_x=el['D_x'],
                                         D_y=el['D_y'], printer=sp,
                                         warningprinter=sp)))
        elif t == 'wake':
            sl = make_slicer(el['slicer'])
            srcs = [make_source(s) for s in el['sources']]
            out.append(('wake', WakeField(sl, *srcs)))
        elif t == 'probe':
            out.append(('probe', (make_slicer(el['slicer']),
                                  el['statistics'])))
        elif t == 'damper':
            from PyHEADTAIL.feedback.transverse_damper import TransverseDamper
            out.append(('map', TransverseDamper(
                el['dampingrate_x'], el['dampingrate_y'], phase=el['phase'],
                local_beta_function=el['local_beta'], printer=sp)))
        else:
            raise ValueError(t)
    return out


COORDS = ('x', 'xp', 'y', 'yp', 'z', 'dp')


def run_case(name, spec):
    beam = make_beam(spec['beam'])
    rec = {'spec': json.dumps(spec)}
    if 'random_seed' in spec:
        import random
        random.seed(spec['random_seed'])
    for k in COORDS:
        rec['init_' + k] = getattr(beam, k).copy()
    elements = make_elements(spec, beam)
    n_turns = spec['n_turns']
    for turn in range(n_turns):
        for j, (kind, el) in enumerate(elements):
            if kind == 'map':
                el.track(beam)
            elif kind == 'wake':
                el.track(beam)
                if turn in (0, n_turns - 1):
                    ss = el.slice_set_deque[0]
                    p = 't%d_e%d_' % (turn, j)
                    rec[p + 'counts'] = ss.n_macroparticles_per_slice
                    rec[p + 'mean_x'] = ss.mean_x
                    rec[p + 'mean_y'] = ss.mean_y
                    rec[p + 'z_bins'] = ss.z_bins
            elif kind == 'probe':
                slicer, stats = el
                ss = slicer.slice(beam, statistics=stats)
                p = 't%d_e%d_' % (turn, j)
                rec[p + 'idx'] = ss.slice_index_of_particle
                rec[p + 'counts'] = ss.n_macroparticles_per_slice
                rec[p + 'z_bins'] = ss.z_bins
                for st in stats:
                    rec[p + st] = getattr(ss, st)
        if turn in (0, n_turns - 1):
            for k in COORDS:
                rec['t%d_%s' % (turn, k)] = getattr(beam, k).copy()
            rec['t%d_gamma' % turn] = np.float64(beam.gamma)
            rec['t%d_p0' % turn] = np.float64(beam.p0)
            rec['t%d_mean_x' % turn] = np.float64(beam.mean_x())
            rec['t%d_mean_y' % turn] = np.float64(beam.mean_y())
            for st in spec.get('record_bunch_stats', ()):
                rec['t%d_bs_%s' % (turn, st)] = np.float64(getattr(beam, st)())
    np.savez_compressed(os.path.join(HERE, name + '.npz'), **rec)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--ref', required=True,
                    help='PyHEADTAIL source tree (read only)')
    ap.add_argument('--scratch', default='/tmp/phk_refbuild')
    ap.add_argument('cases', nargs='*')
    a = ap.parse_args()
    build_reference(a.ref, a.scratch)
    import PyHEADTAIL  # noqa: F401
    patch_reference_numpy2()
    for name in (a.cases or sorted(C.CASES)):
        run_case(name, C.CASES[name])
        print('wrote', name)


if __name__ == '__main__':
    main()
