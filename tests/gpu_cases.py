"""Build pyheadtail_gb300 objects from a case specification (the schema of
tests/golden/cases.py) and run them -- the GPU counterpart of
oracle/cases.py, with the same record layout."""
import numpy as np
from scipy.constants import e, m_p

from pyheadtail_gb300.general.printers import SilentPrinter
from pyheadtail_gb300.impedances import wakes as W
from pyheadtail_gb300.particles.particles import COORDS, Particles
from pyheadtail_gb300.particles.slicing import UniformBinSlicer
from pyheadtail_gb300.trackers.detuners import AmplitudeDetuning, Chromaticity
from pyheadtail_gb300.trackers.longitudinal_tracking import LinearMap, RFSystems
from pyheadtail_gb300.trackers.transverse_tracking import TransverseMap

SP = SilentPrinter()


def make_beam(bp, coords, precision='fp64'):
    return Particles(len(coords['x']), bp['intensity'] / bp['n'], e, m_p,
                     bp['circumference'], bp['gamma'],
                     coords_n_momenta_dict=coords, precision=precision)


def make_slicer(sp):
    z_cuts = None if sp['z_cuts'] is None else tuple(sp['z_cuts'])
    if sp.get('mode') == 'uniform_charge':
        from pyheadtail_gb300.particles.slicing import UniformChargeSlicer
        return UniformChargeSlicer(sp['n_slices'], n_sigma_z=sp['n_sigma_z'],
                                   z_cuts=z_cuts, warningprinter=SP)
    return UniformBinSlicer(sp['n_slices'], n_sigma_z=sp['n_sigma_z'],
                            z_cuts=z_cuts, warningprinter=SP)


def make_source(src):
    ntw = src['n_turns_wake']
    if src['type'] == 'resonator':
        args = (src['R'], src['f'], src['Q'])
        if src['kind'] == 'circular':
            return W.CircularResonator(*args, n_turns_wake=ntw)
        if src['kind'] == 'parallel_horizontal':
            return W.ParallelHorizontalPlatesResonator(*args, n_turns_wake=ntw)
        if src['kind'] == 'longitudinal':
            return W.Resonator(*args, Yokoya_X1=0, Yokoya_Y1=0, Yokoya_X2=0,
                               Yokoya_Y2=0, switch_Z=True, n_turns_wake=ntw)
    if src['type'] == 'wake_table':
        import os
        path = os.path.join(os.path.dirname(os.path.abspath(__file__)),
                            'golden', src['file'])
        return W.WakeTable(path, src['columns'], n_turns_wake=ntw,
                           printer=SP)
    if src['type'] == 'resistive_wall' and src['kind'] == 'circular':
        return W.CircularResistiveWall(src['b'], src['L'], src['sigma'],
                                       src['dt_min'], n_turns_wake=ntw)
    raise ValueError(src)


def make_elements(spec, beam):
    out = []
    for el in spec['elements']:
        t = el['type']
        if t == 'transverse':
            dets = []
            if el['chroma'] is not None:
                dets.append(Chromaticity(*el['chroma']))
            if el['amplitude'] is not None:
                dets.append(AmplitudeDetuning(*el['amplitude']))
            aq = lambda v: np.array(v) if isinstance(v, list) else v
            tm = TransverseMap(np.array(el['s']), np.array(el['alpha_x']),
                               np.array(el['beta_x']), np.array(el['D_x']),
                               np.array(el['alpha_y']), np.array(el['beta_y']),
                               np.array(el['D_y']), aq(el['accQ_x']),
                               aq(el['accQ_y']), dets, printer=SP)
            out.extend(('map', m) for m in tm)
        elif t == 'rf':
            out.append(('map', RFSystems(
                beam.circumference, el['h'], el['V'], el['dphi'], el['alpha'],
                beam.gamma, p_increment=el['p_increment'], D_x=el['D_x'],
                D_y=el['D_y'], shrink_transverse=el['shrink_transverse'],
                charge=e, mass=m_p, printer=SP, warningprinter=SP)))
        elif t == 'linear_map':
            out.append(('map', LinearMap(el['alpha'], beam.circumference,
                                         el['Q_s'], D_x=el['D_x'],
                                         D_y=el['D_y'], printer=SP,
                                         warningprinter=SP)))
        elif t == 'wake':
            sl = make_slicer(el['slicer'])
            srcs = [make_source(s) for s in el['sources']]
            out.append(('wake', W.WakeField(sl, *srcs)))
        elif t == 'probe':
            out.append(('probe', (make_slicer(el['slicer']),
                                  el['statistics'])))
        elif t == 'damper':
            from pyheadtail_gb300.feedback.transverse_damper import \
                TransverseDamper
            out.append(('map', TransverseDamper(
                el['dampingrate_x'], el['dampingrate_y'], phase=el['phase'],
                local_beta_function=el['local_beta'], printer=SP)))
        else:
            raise ValueError(t)
    return out


def _np(t):
    return t.detach().double().cpu().numpy() if hasattr(t, 'cpu') else t


def run(spec, beam, n_turns=None, record_turns=None):
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
                    ss = el.slice_set_deque[0]
                    rec[p + 'counts'] = ss.n_macroparticles_per_slice.cpu().numpy()
                    rec[p + 'mean_x'] = _np(ss.mean_x)
                    rec[p + 'mean_y'] = _np(ss.mean_y)
                    rec[p + 'z_bins'] = ss.z_bins
            elif kind == 'probe':
                slicer, stats = el
                ss = slicer.slice(beam, statistics=stats)
                rec[p + 'idx'] = ss.slice_index_of_particle.cpu().numpy()
                rec[p + 'counts'] = ss.n_macroparticles_per_slice.cpu().numpy()
                rec[p + 'z_bins'] = ss.z_bins
                for st in stats:
                    rec[p + st] = _np(getattr(ss, st))
        if turn in record_turns:
            # statistics first: they see the wake kicks still pending
            for st in spec.get('record_bunch_stats', ()):
                rec['t%d_bs_%s' % (turn, st)] = np.float64(getattr(beam, st)())
            c = beam.coords_numpy()
            for k in COORDS:
                rec['t%d_%s' % (turn, k)] = c[k]
            rec['t%d_gamma' % turn] = np.float64(beam.gamma)
            rec['t%d_p0' % turn] = np.float64(beam.p0)
            rec['t%d_mean_x' % turn] = np.float64(beam.mean_x())
            rec['t%d_mean_y' % turn] = np.float64(beam.mean_y())
    return rec
