"""FP32 form: per-slice sums are exact fixed-point sums, hence bit-identical
on every launch.

The fused kernel of the precision form accumulates x and y per slice as
integers at a power-of-two scale agreed by each thread-block cluster (the
largest |u| of its first tiles maps to [2^26, 2^27)), so the only error is
the rounding of each value to that scale: at most 2^-27 of the largest
|u| per value, below the FP32 rounding of the value itself.  Checked here:

* at the multi-turn wake workload's size (1e7 macroparticles, 500 slices)
  and at the large single bunch's (5e7, 1000 slices): repeated slicings of
  the same coordinates, and two turns of two beams made from the same
  coordinates, give bit-identical counts, means and coordinates;
* the means equal the FP64 sums of the FP32 values within that bound;
* values far above the scale (exact 64-bit path), NaN and +-inf (the
  slice mean becomes NaN or +-inf as a floating-point sum would), and
  clusters whose first tiles are all zero.
The reference sums each slice sequentially in FP64
(cobra_functions/stats.pyx:235-253)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip('torch')

COORDS = ('x', 'xp', 'y', 'yp', 'z', 'dp')
SIGMAS = (1e-3, 1e-5, 1e-3, 1e-5, 0.23, 1e-3)


def _bits(t):
    return t.contiguous().view(torch.int64)


def _random_coords(n, seed):
    g = torch.Generator(device='cuda').manual_seed(seed)
    return {k: torch.randn(n, dtype=torch.float64, device='cuda',
                           generator=g) * s for k, s in zip(COORDS, SIGMAS)}


def _fp64_means(beam, S, q):
    """Counts and FP64 means of coordinate q of the beam's own FP32 values,
    binned with the reference formula."""
    import cases as C
    tail, head = C.Z_CUTS
    width = (head - tail) / float(S)
    zh = beam.z.double().cpu().numpy()
    idx = np.floor((zh - tail) / width)
    inside = (idx >= 0) & (idx < S)
    k = idx[inside].astype(np.int64)
    u = getattr(beam, q).double().cpu().numpy()[inside]
    counts = np.bincount(k, minlength=S)
    sums = np.bincount(k, weights=u, minlength=S)
    return counts, np.where(counts > 0, sums / np.maximum(counts, 1), 0.)


@pytest.fixture(params=[(-1, -1, -1), (1, -1, -1)],
                ids=['tile_kernel', 'streaming_kernel'])
def plan(request):
    """Launch plan of the FP32 pass (phk_set_track_plan): the default
    tile-shared kernel and the streaming kernel."""
    from pyheadtail_gb300 import _native as N
    N.call('phk_set_track_plan', *request.param)
    yield request.param
    N.call('phk_set_track_plan', -1, -1, -1)


@pytest.mark.parametrize('n,S', [(10**7, 500), (5 * 10**7, 1000)])
def test_repeated_slicing_bit_identical_and_exact(n, S, plan):
    import gpu_cases as G
    import cases as C
    beam = G.make_beam(C.beam_params(n, 0), _random_coords(n, 0),
                       precision='fp32')
    sl = G.make_slicer(C.slicer(S))
    runs = []
    for _ in range(3):
        ss = sl.slice(beam, statistics=['mean_x', 'mean_y'])
        runs.append((ss.n_macroparticles_per_slice.clone(),
                     ss.mean_x.clone(), ss.mean_y.clone()))
        beam.clean_slices()
    for c, mx, my in runs[1:]:
        assert torch.equal(c, runs[0][0])
        assert torch.equal(_bits(mx), _bits(runs[0][1]))
        assert torch.equal(_bits(my), _bits(runs[0][2]))
    for q, got in (('x', runs[0][1]), ('y', runs[0][2])):
        counts, mean = _fp64_means(beam, S, q)
        np.testing.assert_array_equal(runs[0][0].cpu().numpy(), counts)
        # per value at most 2^-27 of the cluster's largest |u|, which is
        # at most the bunch's largest |u|
        umax = float(getattr(beam, q).abs().max())
        err = np.max(np.abs(got.cpu().numpy() - mean))
        assert err <= 2.0**-27 * umax * (1 + 1e-9), (q, err, umax)


def test_turns_of_two_equal_beams_bit_identical(plan):
    """Two turns of the large-bunch physics (Q' = 2, amplitude detuning,
    RF, 1000 slices, resonator + 50-turn resistive wall) on two beams made
    from the same coordinates: identical slice sums and coordinates."""
    import gpu_cases as G
    import cases as C
    n = 2 * 10**6
    coords = _random_coords(n, 4)
    spec = dict(beam=C.beam_params(n, 4), n_turns=2, elements=[
        C.smooth_transverse(chroma=[2., 2.],
                            amplitude=[1e-11, 1e-11, -5e-12]),
        C.rf(), C.wake(C.slicer(1000), C.resonator(),
                       C.resistive_wall(n_turns_wake=50))])
    recs = []
    for _ in range(2):
        beam = G.make_beam(spec['beam'], coords, precision='fp32')
        recs.append(G.run(spec, beam, n_turns=2))
    for k, v in recs[0].items():
        a = np.atleast_1d(np.asarray(v))
        b = np.atleast_1d(np.asarray(recs[1][k]))
        assert a.dtype == b.dtype and a.shape == b.shape, k
        assert a.tobytes() == b.tobytes(), k


def _slice_and_reference(coords, n, S):
    import gpu_cases as G
    import cases as C
    beam = G.make_beam(C.beam_params(n, 7), coords, precision='fp32')
    sl = G.make_slicer(C.slicer(S))
    ss = sl.slice(beam, statistics=['mean_x', 'mean_y'])
    tail, head = C.Z_CUTS
    width = (head - tail) / float(S)
    xf = beam.x.double().cpu().numpy()
    zf = beam.z.double().cpu().numpy()
    idx = np.floor((zf - tail) / width)
    with np.errstate(invalid='ignore'):
        want = np.array([xf[idx == s].mean() if np.any(idx == s) else 0.
                         for s in range(S)])
    counts = np.bincount(idx[(idx >= 0) & (idx < S)].astype(np.int64),
                         minlength=S)
    np.testing.assert_array_equal(ss.n_macroparticles_per_slice.cpu().numpy(),
                                  counts)
    return ss.mean_x.cpu().numpy(), want, xf


def test_outliers_nan_and_inf():
    """Values up to 2^14 times the largest |x| of the cluster's first tiles
    take the exact 64-bit path; NaN and infinities make the slice mean NaN
    / +-inf as a floating-point sum would (slice 20: NaN, 21: +inf, 22:
    both infinities, 23: -inf)."""
    import cases as C
    # several tiles per CTA: the last (partial) tile, which holds the
    # planted values, belongs to a CTA whose first tile is ordinary
    n, S = 2 * 10**6 + 300, 50
    rng = np.random.RandomState(7)
    tail, head = C.Z_CUTS
    width = (head - tail) / float(S)
    centers = tail + (np.arange(S) + 0.5) * width
    z = rng.normal(0, 0.23, n)
    x = rng.normal(0, 1e-3, n)
    z[-10:] = centers[10]
    x[-10:] = [0.3, -0.7, 1.25, 5e-2, -4.0, 9.0, 2.5e-1, -1e-1, 6.0, 10.0]
    z[-20:-10] = centers[[20, 21, 22, 22, 23, 20, 21, 22, 23, 23]]
    x[-20:-10] = [np.nan, np.inf, np.inf, -np.inf, -np.inf,
                  1e-3, 2e-3, 3e-3, 4e-3, 5e-3]
    coords = dict(x=x, xp=rng.normal(0, 1e-5, n), y=rng.normal(0, 1e-3, n),
                  yp=rng.normal(0, 1e-5, n), z=z, dp=rng.normal(0, 1e-3, n))
    got, want, xf = _slice_and_reference(coords, n, S)
    assert np.isnan(got[20]) and np.isnan(want[20])
    assert got[21] == np.inf and want[21] == np.inf
    assert np.isnan(got[22]) and np.isnan(want[22])
    assert got[23] == -np.inf and want[23] == -np.inf
    ok = np.isfinite(want)
    ok[10] = False
    typical = np.max(np.abs(xf[:-20]))
    assert np.max(np.abs(got[ok] - want[ok])) <= 2.0**-27 * typical
    # the outliers themselves are exact: only the ordinary values round
    assert abs(got[10] - want[10]) <= 2.0**-27 * typical


def test_zero_first_tiles():
    """Every CTA's first tile holds x = 0 (no scale from the data): the
    clusters fall back to the scale 2^40, the later values take the exact
    levels."""
    n, S = 2 * 10**6, 100
    rng = np.random.RandomState(8)
    x = rng.normal(0, 1e-3, n)
    x[:600 * 512] = 0.0
    coords = dict(x=x, xp=rng.normal(0, 1e-5, n), y=rng.normal(0, 1e-3, n),
                  yp=rng.normal(0, 1e-5, n), z=rng.normal(0, 0.23, n),
                  dp=rng.normal(0, 1e-3, n))
    got, want, xf = _slice_and_reference(coords, n, S)
    assert np.max(np.abs(got - want)) <= 2.0**-40
