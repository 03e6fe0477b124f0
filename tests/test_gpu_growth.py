"""Transverse instability growth rate of the multi-turn wake workload
(resonator + 50-turn resistive wall, 500 slices, RF h=4620, Q'=0) at 1e5
macroparticles over 2000 turns: plain FP64 GPU form and FP32 precision form
against the FP64 oracle on the same seeded bunch.

The growth rate is measured as the reference's simulation test does it
(tests/simulation_tests/test_bb_resonator.py:99-106): Hilbert envelope of
the turn-by-turn centroid, linear regression of its logarithm over the
second half of the run.  Bars: FP64 within 1e-6 relative of the oracle,
FP32 within 1 %.  Fixed cuts at +-3 sigma_z keep the FP32 form on the
tensor-core wake."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip('torch')
scipy_signal = pytest.importorskip('scipy.signal')
scipy_stats = pytest.importorskip('scipy.stats')

N_TURNS = 2000


def growth_rate(centroid, first=N_TURNS // 2):
    env = np.abs(scipy_signal.hilbert(centroid))
    turns = np.arange(len(centroid))
    fit = scipy_stats.linregress(turns[first:], np.log(env[first:]))
    return fit.slope


def _spec():
    import cases as C
    return dict(beam=C.beam_params(100000, 2), n_turns=N_TURNS, elements=[
        C.smooth_transverse(), C.rf(),
        C.wake(C.slicer(500), C.resonator(),
               C.resistive_wall(n_turns_wake=50))])


def _oracle_centroids(spec):
    from oracle import cases as OC
    beam = OC.make_beam(spec['beam'])
    els = [el for _, el in OC.make_elements(spec, beam)]
    cx = np.zeros(N_TURNS)
    cy = np.zeros(N_TURNS)
    for t in range(N_TURNS):
        for el in els:
            el.track(beam)
        cx[t], cy[t] = beam.mean_x(), beam.mean_y()
    return cx, cy, OC.make_beam(spec['beam']).coords()


def _gpu_centroids(spec, coords, precision):
    import gpu_cases as G
    beam = G.make_beam(spec['beam'], coords, precision=precision)
    els = [el for _, el in G.make_elements(spec, beam)]
    cx = torch.zeros(N_TURNS, dtype=torch.float64, device='cuda')
    cy = torch.zeros(N_TURNS, dtype=torch.float64, device='cuda')
    for t in range(N_TURNS):
        for el in els:
            el.track(beam)
        beam._engine.sync_for('x')
        cx[t] = beam._c['x'].double().mean()
        cy[t] = beam._c['y'].double().mean()
    return cx.cpu().numpy(), cy.cpu().numpy()


def test_growth_rate_fp64_and_fp32_against_oracle():
    spec = _spec()
    ox, oy, coords = _oracle_centroids(spec)
    g_ref = (growth_rate(ox), growth_rate(oy))
    assert g_ref[0] > 1e-3 and g_ref[1] > 1e-4, g_ref   # unstable: measurable
    for precision, tol in (('fp64', 1e-6), ('fp32', 1e-2)):
        gx, gy = _gpu_centroids(spec, coords, precision)
        g = (growth_rate(gx), growth_rate(gy))
        for plane in range(2):
            rel = abs(g[plane] - g_ref[plane]) / g_ref[plane]
            print('growth %s plane %d: %.6e vs oracle %.6e (rel %.2e)'
                  % (precision, plane, g[plane], g_ref[plane], rel))
            assert rel <= tol, (precision, plane, g, g_ref)
