"""Errors of the FP32 precision form against the FP64 oracle, on C2 physics
(Q'=5, amplitude detuning, RF h=4620, 200 slices, resonator) at 1e5
macroparticles, with a probe slicing of 50 slices that reports per-slice
centroids and emittances.

The precision form stores the coordinates in FP32, keeps the phase
arguments at FP64-class precision (float-float) with an unbiased sin/cos,
bins the FP32 z with the reference formula and accumulates the slice sums
to better than the FP32 rounding of their terms.  Its errors against the
FP64 oracle come from two sources inherent to the form: the FP32 rounding
of the stored coordinates every turn, which the strong amplitude detuning
of this lattice turns into phase errors (rounding only the initial bunch
already moves the FP64 oracle's coordinates by 1.3e-6 RMS, 4e-5 at most
after 30 turns), and particles whose FP32 z rounds across a slice edge,
which move part of a slice's dipole moment to its neighbour and so change
the wake kicks.  Measured on a GB300 after 30 turns (relative to the RMS of
the quantity): coordinates 3.1e-5 RMS, 7.9e-3 for the worst particle; slice
dipole moments (count x centroid, what the wake sees) 8.3e-2 at the
worst slice (one particle crossing moves ~4 % of a slice's moment); per-slice
normalised emittances 9.4e-6; bunch centroid 1.1e-7.  The bars are about
three times these."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip('torch')

COORDS = ('x', 'xp', 'y', 'yp', 'z', 'dp')
STATS = ['mean_x', 'mean_y', 'sigma_x', 'epsn_x', 'epsn_y', 'epsn_z']
T = 30
BARS = {'coords_rms': 1e-4, 'coords_max': 3e-2, 'slice_moment': 0.25,
        'slice_emittance': 3e-5, 'bunch_centroid': 1e-6}


def _errors():
    import cases as C
    import gpu_cases as G
    from oracle import cases as OC
    spec = dict(C.CASES['c2_full'])
    spec['beam'] = C.beam_params(100000, 1)
    spec['elements'] = list(spec['elements']) + [C.probe(C.slicer(50), STATS)]
    ob = OC.make_beam(spec['beam'])
    coords = ob.coords()
    ref = OC.run(spec, ob, n_turns=T, record_turns=(T - 1,))
    beam = G.make_beam(spec['beam'], coords, precision='fp32')
    rec = G.run(spec, beam, n_turns=T, record_turns=(T - 1,))
    kinds = [k for k, _ in G.make_elements(spec, beam)]
    wake_j, probe_j = kinds.index('wake'), len(kinds) - 1
    t = 't%d_' % (T - 1)
    e = {}
    rel = []
    for k in COORDS:
        g, r = np.asarray(rec[t + k], np.float64), ref[t + k]
        rel.append(np.abs(g - r) / np.sqrt(np.mean(r**2)))
    rel = np.concatenate(rel)
    e['coords_rms'] = float(np.sqrt(np.mean(rel**2)))
    e['coords_max'] = float(rel.max())

    def rms_rel(g, r):
        g, r = np.asarray(g, np.float64), np.asarray(r, np.float64)
        ok = np.isfinite(r) & np.isfinite(g)
        return float(np.max(np.abs(g[ok] - r[ok])) / np.sqrt(np.mean(r[ok]**2)))
    w = '%se%d_' % (t, wake_j)
    e['slice_moment'] = max(
        rms_rel(np.asarray(rec[w + 'counts'], np.float64) * rec[w + q],
                ref[w + 'counts'] * ref[w + q])
        for q in ('mean_x', 'mean_y'))
    pe = []
    for q in ('epsn_x', 'epsn_y', 'epsn_z'):
        g = np.asarray(rec['%se%d_%s' % (t, probe_j, q)], np.float64)
        r = np.asarray(ref['%se%d_%s' % (t, probe_j, q)], np.float64)
        ok = np.isfinite(r) & (r > 0)
        pe.append(float(np.max(np.abs(g[ok] - r[ok]) / r[ok])))
    e['slice_emittance'] = max(pe)
    e['bunch_centroid'] = max(
        float(abs(rec[t + q] - ref[t + q]) / np.sqrt(np.mean(ref[t + q[5:]]**2)))
        for q in ('mean_x', 'mean_y'))
    return e


# launch plans of the FP32 pass (phk_set_track_plan: variant, ring
# stages, shared-memory budget in KB): the default, the streaming kernel,
# and the tile-shared kernel with fixed stages and a larger budget
PLANS = [(-1, -1, -1), (1, -1, -1), (1, 4, 96), (0, 2, 72), (0, 0, -1)]


@pytest.mark.parametrize('plan', PLANS, ids=lambda p: 'plan%d_%d_%d' % p)
def test_fp32_form_errors_against_fp64_oracle(plan):
    from pyheadtail_gb300 import _native as N
    N.call('phk_set_track_plan', *plan)
    try:
        e = _errors()
    finally:
        N.call('phk_set_track_plan', -1, -1, -1)
    print('FP32 form errors after %d turns, plan %s: %s' % (T, plan, e))
    for k, bar in BARS.items():
        assert e[k] <= bar, (k, e)
