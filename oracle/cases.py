"""Build and run oracle objects from a case specification dict (the schema
of ``tests/golden/cases.py``).  Test infrastructure only."""
import os

import numpy as np
from scipy.constants import e, m_p

from . import turn_loop as T


def make_beam(bp, coords=None):
    """Seeded bunch (or the given coordinates) with the case's scalars."""
    if coords is None:
        return T.gaussian_bunch(bp['n'], bp['seed'], bp['gamma'], m_p, e,
                                bp['circumference'], bp['intensity'],
                                bp['epsn_x'], bp['epsn_y'], bp['beta_x'],
                                bp['beta_y'], bp['sigma_z'], bp['sigma_dp'],
                                bp['alpha_x'], bp['alpha_y'])
    return T.Beam(coords, bp['intensity'] / bp['n'], e, m_p,
                  bp['circumference'], bp['gamma'])


def table_path(name):
    """Wake tables of the cases live beside the golden fixtures."""
    return os.path.join(os.path.dirname(os.path.dirname(
        os.path.abspath(__file__))), 'tests', 'golden', name)


def make_slicer(sp):
    z_cuts = None if sp['z_cuts'] is None else tuple(sp['z_cuts'])
    cls = (T.UniformChargeSlicer if sp.get('mode') == 'uniform_charge'
           else T.UniformBinSlicer)
    return cls(sp['n_slices'], n_sigma_z=sp['n_sigma_z'], z_cuts=z_cuts)


def make_kicks(src, slicer):
    """WakeSource.get_wake_kicks order: X1 dipole, X2 quad, Y1 dipole,
    Y2 quad, Z constant (wakes.py:402-441)."""
    ntw = src['n_turns_wake']
    if src['type'] == 'resonator':
        R, f, Q = src['R'], src['f'], src['Q']
        yok = {'circular': (1., 1., 0., 0., False),
               'parallel_horizontal': (np.pi**2 / 24., np.pi**2 / 12.,
                                       -np.pi**2 / 24., np.pi**2 / 24., False),
               'longitudinal': (0, 0, 0, 0, True)}[src['kind']]
        X1, Y1, X2, Y2, Z = yok
        kicks = []
        if X1:
            kicks.append(T.WakeKick(T.resonator_transverse(R, f, Q, X1),
                                    slicer, ntw, 'xp', 'x'))
        if X2:
            kicks.append(T.WakeKick(T.resonator_transverse(R, f, Q, X2),
                                    slicer, ntw, 'xp', None, quad='x'))
        if Y1:
            kicks.append(T.WakeKick(T.resonator_transverse(R, f, Q, Y1),
                                    slicer, ntw, 'yp', 'y'))
        if Y2:
            kicks.append(T.WakeKick(T.resonator_transverse(R, f, Q, Y2),
                                    slicer, ntw, 'yp', None, quad='y'))
        if Z:
            kicks.append(T.WakeKick(T.resonator_longitudinal(R, f, Q),
                                    slicer, ntw, 'dp', None))
        return kicks
    if src['type'] == 'wake_table':
        table = T.load_wake_table(table_path(src['file']), src['columns'])
        kicks = []
        for name, target, moment, quad in T.TABLE_KICKS:
            if name not in table:
                continue
            wf = (T.table_longitudinal(table) if name == 'longitudinal'
                  else T.table_transverse(table, name))
            kicks.append(T.WakeKick(wf, slicer, ntw, target, moment,
                                    quad=quad))
        return kicks
    if src['type'] == 'resistive_wall':
        wf = T.resistive_wall_transverse(src['b'], src['L'], src['sigma'],
                                         src['dt_min'], 1.)
        return [T.WakeKick(wf, slicer, ntw, 'xp', 'x'),
                T.WakeKick(wf, slicer, ntw, 'yp', 'y')]
    raise ValueError(src)


def make_elements(spec, beam):
    out = []
    for el in spec['elements']:
        t = el['type']
        if t == 'transverse':
            accQ_x = (np.array(el['accQ_x']) if isinstance(el['accQ_x'], list)
                      else el['accQ_x'])
            accQ_y = (np.array(el['accQ_y']) if isinstance(el['accQ_y'], list)
                      else el['accQ_y'])
            segs = T.transverse_map(
                el['s'], np.array(el['alpha_x']), np.array(el['beta_x']),
                np.array(el['D_x']), np.array(el['alpha_y']),
                np.array(el['beta_y']), np.array(el['D_y']), accQ_x, accQ_y,
                chroma=el['chroma'], amplitude=el['amplitude'])
            out.extend(('map', s) for s in segs)
        elif t == 'rf':
            out.append(('map', T.RFSystems(
                beam.circumference, el['h'], el['V'], el['dphi'], el['alpha'],
                beam.gamma, p_increment=el['p_increment'], D_x=el['D_x'],
                D_y=el['D_y'], shrink_transverse=el['shrink_transverse'],
                charge=e, mass=m_p)))
        elif t == 'linear_map':
            out.append(('map', T.LinearMap(el['alpha'], beam.circumference,
                                           el['Q_s'], D_x=el['D_x'],
                                           D_y=el['D_y'])))
        elif t == 'wake':
            sl = make_slicer(el['slicer'])
            kicks = []
            for s in el['sources']:
                kicks.extend(make_kicks(s, sl))
            nmax = max(s['n_turns_wake'] for s in el['sources'])
            out.append(('wake', T.WakeField(sl, kicks, nmax)))
        elif t == 'probe':
            out.append(('probe', (make_slicer(el['slicer']),
                                  el['statistics'])))
        elif t == 'damper':
            out.append(('map', T.TransverseDamper(
                el['dampingrate_x'], el['dampingrate_y'], el['phase'],
                el['local_beta'])))
        else:
            raise ValueError(t)
    return out


def run(spec, beam, n_turns=None, record_turns=None):
    """Track ``beam`` through the case; return the fixture-shaped record."""
    if 'random_seed' in spec:
        import random
        random.seed(spec['random_seed'])
    elements = make_elements(spec, beam)
    n_turns = spec['n_turns'] if n_turns is None else n_turns
    if record_turns is None:
        record_turns = (0, n_turns - 1)
    rec = {}
    for turn in range(n_turns):
        for j, (kind, el) in enumerate(elements):
            p = 't%d_e%d_' % (turn, j)
            if kind == 'map':
                el.track(beam)
            elif kind == 'wake':
                el.track(beam)
                if turn in record_turns:
                    ss = el.slice_sets[0]
                    rec[p + 'counts'] = ss.n_macroparticles_per_slice
                    rec[p + 'mean_x'] = ss.mean_x
                    rec[p + 'mean_y'] = ss.mean_y
                    rec[p + 'z_bins'] = ss.z_bins
            elif kind == 'probe':
                slicer, stats = el
                ss = slicer.slice(beam, statistics=stats)
                rec[p + 'idx'] = ss.slice_index_of_particle
                rec[p + 'counts'] = ss.n_macroparticles_per_slice
                rec[p + 'z_bins'] = ss.z_bins
                for st in stats:
                    rec[p + st] = getattr(ss, st)
        if turn in record_turns:
            for k in T.Beam.COORDS:
                rec['t%d_%s' % (turn, k)] = getattr(beam, k).copy()
            rec['t%d_gamma' % turn] = np.float64(beam.gamma)
            rec['t%d_p0' % turn] = np.float64(beam.p0)
            rec['t%d_mean_x' % turn] = np.float64(beam.mean_x())
            rec['t%d_mean_y' % turn] = np.float64(beam.mean_y())
            for st in spec.get('record_bunch_stats', ()):
                rec['t%d_bs_%s' % (turn, st)] = np.float64(getattr(beam, st)())
    return rec
