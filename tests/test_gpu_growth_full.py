"""Instability growth rate of the multi-turn wake workload at its full size:
1e7 macroparticles, 500 slices, resonator + 50-turn resistive wall, RF
h=4620, Q'=0, 2000 turns, in the plain FP64 form and the FP32 precision
form, against the centroid trace that PyHEADTAIL itself produced on the
same seeded bunch (tests/golden/growth/c3_1e7.npz, written by
tests/golden/make_golden_c3_growth.py).

The loop is the reference test's (tests/simulation_tests/
test_bb_resonator.py:91-96: every element's track, then bunch.mean_x() /
mean_y()), and so is the growth rate: Hilbert envelope of the centroid,
linear fit of its logarithm, here over the second half of the run.  Bars:
the precision form's growth rate within 1 % of the reference's (the target
the form is built for); the plain form's within 1e-6 relative, and its
centroid trace within 1e-6 of the trace's RMS."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip('torch')
scipy_signal = pytest.importorskip('scipy.signal')
scipy_stats = pytest.importorskip('scipy.stats')

FIXTURE = os.path.join(os.path.dirname(__file__), 'golden', 'growth',
                       'c3_1e7.npz')
N_TURNS = 2000


def growth_rate(centroid, first=N_TURNS // 2):
    env = np.abs(scipy_signal.hilbert(centroid))
    turns = np.arange(len(centroid))
    return scipy_stats.linregress(turns[first:], np.log(env[first:])).slope


@pytest.fixture(scope='module')
def reference():
    if not os.path.exists(FIXTURE):
        pytest.skip('growth fixture not generated')
    with np.load(FIXTURE) as f:
        return {k: f[k] for k in f.files}


@pytest.fixture(scope='module')
def setup():
    import cases as C
    from oracle import cases as OC
    spec = dict(beam=C.beam_params(10**7, 2), n_turns=N_TURNS, elements=[
        C.smooth_transverse(), C.rf(),
        C.wake(C.slicer(500), C.resonator(),
               C.resistive_wall(n_turns_wake=50))])
    coords = OC.make_beam(spec['beam']).coords()
    return spec, coords


def _trace(spec, coords, precision):
    import gpu_cases as G
    beam = G.make_beam(spec['beam'], coords, precision=precision)
    els = [el for _, el in G.make_elements(spec, beam)]
    mx = np.zeros(N_TURNS)
    my = np.zeros(N_TURNS)
    for t in range(N_TURNS):
        for el in els:
            el.track(beam)
        mx[t], my[t] = beam.mean_x(), beam.mean_y()
    return mx, my


@pytest.mark.parametrize('precision', ['fp64', 'fp32'])
def test_growth_rate_full_size(reference, setup, precision):
    spec, coords = setup
    mx, my = _trace(spec, coords, precision)
    for plane, got, want in (('x', mx, reference['mean_x']),
                             ('y', my, reference['mean_y'])):
        g, r = growth_rate(got), growth_rate(want)
        rel = abs(g - r) / abs(r)
        trace = np.max(np.abs(got - want)) / np.sqrt(np.mean(want**2))
        print('%s %s: growth %.6e vs reference %.6e (rel %.2e), trace '
              'max diff %.2e of its RMS' % (precision, plane, g, r, rel, trace))
        assert r > 1e-3
        if precision == 'fp64':
            assert rel <= 1e-6, (plane, g, r)
            assert trace <= 1e-6, (plane, trace)
        else:
            assert rel <= 1e-2, (plane, g, r)
