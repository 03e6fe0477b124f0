"""Synchrotron assembly on the host (no GPU), against fixtures made by
running the reference's Synchrotron (tests/golden/synchrotron/*.npz):
the one-turn map's element sequence, Q_s, circumference and gamma, and --
for the 'linear' longitudinal mode -- the seeded Gaussian bunch of
generate_6D_Gaussian_bunch bit for bit."""
import json
import os

import numpy as np
import pytest

pytest.importorskip('torch')

GOLDEN = os.path.join(os.path.dirname(__file__), 'golden', 'synchrotron')
COORDS = ('x', 'xp', 'y', 'yp', 'z', 'dp')


def load(name):
    with np.load(os.path.join(GOLDEN, name + '.npz')) as f:
        return {k: f[k] for k in f.files}


def build(spec):
    """Our Synchrotron with the spec's extras; returns the machine."""
    from scipy.constants import e, m_p
    import cases as C
    from pyheadtail_gb300.feedback.transverse_damper import TransverseDamper
    from pyheadtail_gb300.general.printers import SilentPrinter
    from pyheadtail_gb300.impedances.wakes import CircularResonator, WakeField
    from pyheadtail_gb300.machines.synchrotron import Synchrotron
    from pyheadtail_gb300.particles.slicing import UniformBinSlicer
    sp = SilentPrinter()
    kw = dict(spec['machine'])
    for k in ('s', 'alpha_x', 'beta_x', 'D_x', 'alpha_y', 'beta_y', 'D_y',
              'accQ_x', 'accQ_y'):
        if isinstance(kw.get(k), list):
            kw[k] = np.array(kw[k])
    machine = Synchrotron(charge=e, mass=m_p, printer=sp, **kw)
    if spec['damper_after_segments']:
        dx, dy = spec['damper_after_segments']
        machine.install_after_each_transverse_segment(
            TransverseDamper(dx, dy, printer=sp))
    if spec['wake']:
        w = spec['wake']
        machine.one_turn_map.append(WakeField(
            UniformBinSlicer(w['n_slices'], z_cuts=tuple(C.Z_CUTS),
                             warningprinter=sp),
            CircularResonator(w['R'], w['f'], w['Q'])))
    return machine


@pytest.mark.parametrize('name', ['synchrotron_linear',
                                  'synchrotron_nonlinear'])
def test_assembly_matches_reference(name):
    g = load(name)
    spec = json.loads(str(g['spec']))
    machine = build(spec)
    assert [type(m).__name__ for m in machine.one_turn_map] == \
        list(g['elements'])
    assert machine.Q_s == g['Q_s']
    assert machine.circumference == g['circumference']
    assert machine.gamma == g['gamma']


def test_linear_mode_bunch_matches_reference_generator():
    g = load('synchrotron_linear')
    spec = json.loads(str(g['spec']))
    machine = build(spec)
    b = spec['bunch']
    np.random.seed(b['seed'])
    coords = machine.gaussian_generator(
        b['n'], b['intensity'], b['epsn_x'], b['epsn_y'],
        b['sigma_z']).coordinates()
    for k in COORDS:
        np.testing.assert_array_equal(coords[k], g['init_' + k], err_msg=k)


def test_unsupported_set_ups_raise():
    g = load('synchrotron_nonlinear')
    spec = json.loads(str(g['spec']))
    machine = build(spec)
    with pytest.raises(NotImplementedError):
        machine.generate_6D_Gaussian_bunch_matched(100, 1e11, 2e-6, 2e-6, 0.2)
    with pytest.raises(NotImplementedError):
        machine.gaussian_generator(100, 1e11, 2e-6, 2e-6, 0.2)
    kw = dict(spec['machine'])
    kw['optics_mode'] = 'smooth'
    with pytest.raises(ValueError):
        build(dict(spec, machine=kw))
