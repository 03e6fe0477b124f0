"""Parity of the plain FP64 GPU path with the reference.

* every golden fixture (made by running PyHEADTAIL itself) is replayed on
  the GPU from the same initial coordinates: slice indices, counts and beam
  scalars bit-exact, coordinates and slice means within 1e-12 relative to
  the coordinate's RMS;
* the C1 workload at its full size (1e5 macroparticles, 100 turns) and the
  C2, multi-turn wake and large-bunch physics at reduced size over 100
  turns are compared with the oracle (the oracle is bit-identical to the
  reference on the fixtures);
* at full workload sizes, the GPU slice index of every particle is checked
  bit for bit against the reference formula evaluated by torch on the GPU
  coordinates.
"""
import glob
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip('torch')

GOLDEN = os.path.join(os.path.dirname(__file__), 'golden')
FIXTURES = sorted(glob.glob(os.path.join(GOLDEN, '*.npz')))
COORDS = ('x', 'xp', 'y', 'yp', 'z', 'dp')
RTOL = 1e-12        # coordinates / slice means, relative to the RMS


def rms_err(got, ref):
    got = np.asarray(got, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    scale = np.sqrt(np.mean(ref**2)) if ref.size else 1.
    if scale == 0:
        scale = 1.
    return float(np.max(np.abs(got - ref)) / scale) if ref.size else 0.


def dynamic_cuts(spec):
    """True if a slicer of the case derives its cuts from the bunch
    (n_sigma_z: mean and sigma of z; the reference sums them sequentially,
    the GPU in a tree, so the cuts agree to ~1e-15 only)."""
    sls = [el['slicer'] for el in spec['elements'] if 'slicer' in el]
    return any(s['z_cuts'] is None and s['n_sigma_z'] for s in sls)


def rms_rel(got, ref):
    """||got - ref||_2 / ||ref||_2."""
    got = np.asarray(got, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    den = np.sqrt(np.mean(ref**2)) if ref.size else 1.
    return float(np.sqrt(np.mean((got - ref)**2)) / (den or 1.))


def compare(rec, ref, label, rtol=RTOL, stat_rtol=1e-9, emit_rtol=1e-7,
            bins_rtol=0.0, sens=None):
    """Emittances per slice are sqrt(s11 s22 - s12^2) of covariances summed
    in a different order than the reference's sequential loop; for slices
    with few particles the determinant cancels by several orders, so they
    get emit_rtol (the sums themselves agree to ~1e-15).  Bin edges are
    bit-exact unless bins_rtol > 0 (dynamic cuts).

    Long runs pass `sens`: for each recorded coordinate (and slice mean),
    how far the oracle itself moves -- worst particle relative to the RMS,
    and RMS-relative -- when its initial coordinates are changed by one
    ulp.  Amplitude detuning, the RF nonlinearity and particles crossing
    slice edges amplify such differences (after 100 turns of the C2
    physics at 2e4: worst particle 5e-12, RMS 1.7e-13; of the large-bunch
    physics with 1000 slices: dp 1.7e-10 and 1.2e-12), so a long run
    checks both norms against rtol or four times the oracle's own
    sensitivity, whichever is larger."""
    for k, v in ref.items():
        if not k.startswith('t'):
            continue
        assert k in rec, '%s: missing %s' % (label, k)
        g = rec[k]
        if '_bs_' in k:
            compare_bunch_stat(rec, ref, k, label)
            continue
        if k.endswith('_z_bins') and bins_rtol > 0:
            np.testing.assert_allclose(g, v, rtol=0, atol=bins_rtol *
                                       np.max(np.abs(v)), err_msg=k)
        elif k.endswith(('_idx', '_counts', '_gamma', '_p0', '_z_bins')):
            np.testing.assert_array_equal(np.asarray(g), v,
                                          err_msg='%s %s' % (label, k))
        elif k.endswith(('_mean_x', '_mean_y')) and np.ndim(v) == 0:
            tol = 1e-12 * max(abs(v), 1e-30) + 1e-18
            if sens is not None and k in sens:
                tol = max(tol, 4 * sens[k][0])
            assert abs(g - v) <= tol, (label, k, g, v, tol)
        elif any(k.endswith('_' + c) for c in COORDS) and np.ndim(v) == 1 \
                and len(k.split('_')) == 2:
            e = rms_err(g, v)
            if sens is None:
                assert e <= rtol, '%s %s: rel err %.3g' % (label, k, e)
            else:
                er = rms_rel(g, v)
                bound = max(rtol, 4 * sens[k][1])
                assert er <= bound, '%s %s: rms rel err %.3g > %.3g' % (
                    label, k, er, bound)
                bound = max(rtol, 4 * sens[k][0])
                assert e <= bound, '%s %s: worst particle %.3g > %.3g' % (
                    label, k, e, bound)
        else:
            # per-slice statistics: skip slices where the reference itself
            # is not finite (sqrt of a negative determinant)
            v = np.asarray(v, dtype=np.float64)
            g = np.asarray(g, dtype=np.float64)
            ok = np.isfinite(v)
            # a slice with no more particles than coordinates in the
            # emittance (x, x' and dp with dispersion; two without) has a
            # singular covariance: its emittance is zero up to rounding,
            # whose sign decides between a tiny value and NaN, on the GPU
            # as in the reference -- only required to be tiny or NaN
            if 'epsn' in k:
                dim = 2 if (k.endswith('eff_epsn_x') or k.endswith('eff_epsn_y')
                            or k.endswith('epsn_z')) else 3
                turn, elem = k.split('_')[:2]
                cnt = np.asarray(ref['%s_%s_counts' % (turn, elem)])
                few = cnt <= dim
                scale = np.max(np.abs(v[ok & ~few])) if np.any(ok & ~few) else 1.
                gf = g[few]
                assert np.all(~np.isfinite(gf) | (np.abs(gf) <= 1e-3 * scale)), \
                    (label, k, gf)
                ok &= ~few
            tol = (rtol if 'mean' in k else
                   emit_rtol if 'epsn' in k else stat_rtol)
            e = rms_err(g[ok], v[ok])
            if sens is not None and k in sens:
                er = rms_rel(g[ok], v[ok])
                assert er <= max(tol, 4 * sens[k][1]), \
                    '%s %s: rms rel err %.3g' % (label, k, er)
                tol = max(tol, 4 * sens[k][0])
            assert e <= tol, '%s %s: rel err %.3g' % (label, k, e)


# bunch statistics (Particles.mean_* ... gamma_Twiss_*): the GPU sums in a
# tree what the reference sums sequentially (np.mean pairwise), so they
# agree to rounding; centroids are compared relative to the spread of the
# coordinate, since a centroid near zero has no relative precision
BUNCH_STAT_RTOL = 1e-12


def compare_bunch_stat(rec, ref, k, label, rtol=BUNCH_STAT_RTOL):
    g, v = float(rec[k]), float(ref[k])
    turn, name = k.split('_bs_')
    scale = abs(v)
    if name.startswith('mean_'):
        scale = max(scale, float(ref['%s_bs_sigma_%s' % (turn, name[5:])]))
    assert abs(g - v) <= rtol * scale, '%s %s: %r vs %r' % (label, k, g, v)


def load(path):
    with np.load(path) as f:
        return {k: f[k] for k in f.files}


@pytest.fixture(scope='module')
def lib():
    from pyheadtail_gb300 import _native
    return _native.load()


@pytest.mark.parametrize('path', FIXTURES,
                         ids=[os.path.basename(p)[:-4] for p in FIXTURES])
def test_golden_fixture_fp64(lib, path):
    import gpu_cases as G
    ref = load(path)
    spec = json.loads(str(ref['spec']))
    coords = {k: ref['init_' + k] for k in COORDS}
    beam = G.make_beam(spec['beam'], coords)
    rec = G.run(spec, beam)
    compare(rec, ref, os.path.basename(path),
            bins_rtol=1e-13 if dynamic_cuts(spec) else 0.0)


def _oracle_vs_gpu(spec, n_turns, record_turns=None, sensitivity=False):
    """GPU and oracle records of the case; with sensitivity=True also the
    oracle's own change (worst particle relative to the RMS, RMS-relative)
    per recorded coordinate and slice mean when its initial coordinates
    move by one ulp."""
    import gpu_cases as G
    from oracle import cases as OC
    obeam = OC.make_beam(spec['beam'])
    coords = obeam.coords()
    ref = OC.run(spec, obeam, n_turns=n_turns, record_turns=record_turns)
    beam = G.make_beam(spec['beam'], coords)
    rec = G.run(spec, beam, n_turns=n_turns, record_turns=record_turns)
    if not sensitivity:
        return rec, ref
    moved = {k: np.nextafter(v, np.inf) for k, v in coords.items()}
    alt = OC.run(spec, OC.make_beam(spec['beam'], moved), n_turns=n_turns,
                 record_turns=record_turns)
    sens = {k: (rms_err(alt[k], ref[k]), rms_rel(alt[k], ref[k])) for k in ref
            if (any(k.endswith('_' + c) for c in COORDS)
                and np.ndim(ref[k]) == 1 and len(k.split('_')) == 2)
            or k.endswith(('_mean_x', '_mean_y')) and np.ndim(ref[k]) == 1}
    for k in ref:
        # bunch centroids: absolute change
        if k.endswith(('_mean_x', '_mean_y')) and np.ndim(ref[k]) == 0:
            d = abs(float(alt[k]) - float(ref[k]))
            sens[k] = (d, d)
    return rec, ref, sens


def test_c1_full_size_100_turns(lib):
    """C1: 1e5 macroparticles, seed 0, linear maps, 50 slices, resonator."""
    import cases as C
    spec = dict(C.CASES['c1_full'])
    spec['beam'] = C.beam_params(100000, 0)
    rec, ref = _oracle_vs_gpu(spec, 100)
    compare(rec, ref, 'c1 100 turns')


def test_c2_reduced_size(lib):
    """C2 physics (Q'=5, amplitude detuning, h=4620 RF, 200 slices,
    resonator) at 1e5 macroparticles, 100 turns."""
    import cases as C
    spec = dict(C.CASES['c2_full'])
    spec['beam'] = C.beam_params(100000, 1)
    rec, ref, sens = _oracle_vs_gpu(spec, 100, record_turns=(0, 49, 99),
                                    sensitivity=True)
    compare(rec, ref, 'c2 100 turns', sens=sens)


def test_multiturn_wake_reduced_size(lib):
    """C3 wake model (500 slices, resonator + 50-turn resistive wall, RF
    h=4620, Q'=0) at 2e4 macroparticles over 100 turns (history full after
    50)."""
    import cases as C
    spec = dict(beam=C.beam_params(20000, 2), n_turns=100, elements=[
        C.smooth_transverse(), C.rf(),
        C.wake(C.slicer(500), C.resonator(),
               C.resistive_wall(n_turns_wake=50))])
    rec, ref, sens = _oracle_vs_gpu(spec, 100, record_turns=(0, 49, 99),
                                    sensitivity=True)
    compare(rec, ref, 'multiturn 100 turns', sens=sens)


def test_large_bunch_physics_reduced_size(lib):
    """C5 physics (Q'=2, amplitude detuning as C2, RF h=4620, 1000 slices,
    resonator + 50-turn resistive wall) at 2e4 macroparticles over 100
    turns."""
    import cases as C
    spec = dict(beam=C.beam_params(20000, 4), n_turns=100, elements=[
        C.smooth_transverse(chroma=[2., 2.],
                            amplitude=[1e-11, 1e-11, -5e-12]),
        C.rf(), C.wake(C.slicer(1000), C.resonator(),
                       C.resistive_wall(n_turns_wake=50))])
    rec, ref, sens = _oracle_vs_gpu(spec, 100, record_turns=(0, 49, 99),
                                    sensitivity=True)
    compare(rec, ref, 'large bunch 100 turns', sens=sens)


@pytest.mark.parametrize('n', [1, 2, 3, 5, 1001, 4099])
def test_ragged_sizes(lib, n):
    """Sizes that are not multiples of the vector width or of a tile."""
    import cases as C
    spec = dict(C.CASES['c2_full'])
    spec['beam'] = C.beam_params(n, 5)
    rec, ref = _oracle_vs_gpu(spec, 3)
    compare(rec, ref, 'n=%d' % n)


def test_edges_outside_nan_and_misaligned(lib):
    """Particles exactly on bin edges, just below them, outside the cuts,
    NaN z, and coordinate tensors that are views at an odd offset (not
    16-byte aligned: scalar path)."""
    import gpu_cases as G
    from pyheadtail_gb300 import _engine as E
    import cases as C
    bp = C.beam_params(4000, 7)
    rng = np.random.RandomState(3)
    S, cuts = 40, (-0.69, 0.69)
    width = (cuts[1] - cuts[0]) / float(S)
    edges, _ = E.exact_edges(cuts[0], width, S, E._F64)
    z = rng.normal(0, 0.4, 4000)
    z[:41] = edges
    z[41:82] = np.nextafter(edges, -np.inf)
    z[82] = np.nan
    z[83:90] = [-5., 5., 0.69, -0.69, 1e300, -1e300, 0.]
    coords = dict(x=rng.normal(0, 1e-3, 4000), xp=rng.normal(0, 1e-5, 4000),
                  y=rng.normal(0, 1e-3, 4000), yp=rng.normal(0, 1e-5, 4000),
                  z=z, dp=rng.normal(0, 1e-3, 4000))
    beam = G.make_beam(bp, coords)
    # re-seat every coordinate as a view one element into a larger buffer
    for k in COORDS:
        big = torch.empty(4001, dtype=torch.float64, device='cuda')
        big[1:] = beam._c[k]
        beam._c[k] = big[1:]
    sl = G.make_slicer(C.slicer(S, z_cuts=cuts))
    ss = sl.slice(beam, statistics=['mean_x', 'mean_y'])
    idx = ss.slice_index_of_particle.cpu().numpy()
    with np.errstate(invalid='ignore'):
        want = np.floor((z - cuts[0]) / width)
    want_i = np.where(np.isfinite(want) & (np.abs(want) < 2**31), want,
                      -2**31).astype(np.int64)
    np.testing.assert_array_equal(idx.astype(np.int64), want_i)
    # expected sums from the x86 conversion convention (NumPy on Arm maps
    # NaN to 0 instead, which would put it into slice 0)
    inside = (want_i >= 0) & (want_i < S)
    counts = np.bincount(want_i[inside], minlength=S)
    np.testing.assert_array_equal(ss.n_macroparticles_per_slice.cpu().numpy(),
                                  counts)
    sums = np.bincount(want_i[inside], weights=coords['x'][inside],
                       minlength=S)
    mean = np.where(counts > 0, sums / np.maximum(counts, 1), 0.)
    assert rms_err(ss.mean_x.cpu().numpy(), mean) <= RTOL


def test_all_outside_and_empty_slices(lib):
    import gpu_cases as G
    import cases as C
    n = 777
    coords = {k: np.zeros(n) for k in COORDS}
    coords['z'] = np.full(n, 3.0)
    beam = G.make_beam(C.beam_params(n, 1), coords)
    sl = G.make_slicer(C.slicer(20))
    ss = sl.slice(beam, statistics=['mean_x', 'mean_y'])
    assert int(ss.n_macroparticles_per_slice.sum()) == 0
    assert float(ss.mean_x.abs().sum()) == 0.0
    assert int((ss.slice_index_of_particle >= 0).sum()) == n   # 5 * 20 / 1.38


@pytest.mark.parametrize('precision', ['fp64', 'fp32'])
@pytest.mark.parametrize('n,S', [(10**7, 500), (5 * 10**7, 1000)])
def test_full_size_binning_bit_exact(lib, n, S, precision):
    """C3 / C5 sizes: every particle's slice index equals the reference
    formula int32(floor((z - tail)/width)) evaluated by torch in FP64 on
    the form's own z.  The first particles sit on every slice edge and on
    the 8 representable values either side of it, where the FP32 lookup's
    table-free path must hand over to the edge table."""
    import gpu_cases as G
    import cases as C
    from pyheadtail_gb300 import _engine as E
    torch.manual_seed(0)
    tail, head = C.Z_CUTS
    width = (head - tail) / float(S)
    z = torch.randn(n, dtype=torch.float64, device='cuda') * 0.23
    code = E._F64 if precision == 'fp64' else E._F32
    edges, _ = E.exact_edges(tail, width, S, code)
    near = [edges]
    lo, hi = edges.copy(), edges.copy()
    for _ in range(8):
        lo = np.nextafter(lo, lo.dtype.type(-np.inf))
        hi = np.nextafter(hi, hi.dtype.type(np.inf))
        near += [lo, hi]
    near = np.concatenate(near).astype(np.float64)
    z[:len(near)] = torch.from_numpy(near).cuda()
    coords = {k: torch.zeros(n, dtype=torch.float64, device='cuda')
              for k in COORDS}
    coords['z'] = z
    coords['x'] = torch.randn(n, dtype=torch.float64, device='cuda') * 1e-3
    beam = G.make_beam(C.beam_params(n, 2), coords, precision=precision)
    assert beam.z.dtype == (torch.float64 if code == E._F64 else torch.float32)
    sl = G.make_slicer(C.slicer(S))
    ss = sl.slice(beam, statistics=['mean_x', 'mean_y'])
    idx = ss.slice_index_of_particle
    # NumPy's IEEE division on the host: torch on the GPU divides by a
    # Python scalar as a multiplication by its reciprocal, which differs
    # from the reference formula by one ulp exactly at slice edges
    zh = beam.z.double().cpu().numpy()
    want = torch.from_numpy(
        np.floor((zh - tail) / width).astype(np.int32)).cuda()
    assert torch.equal(idx, want)
    inside = (want >= 0) & (want < S)
    counts = torch.bincount(want[inside].long(), minlength=S).to(torch.int32)
    assert torch.equal(ss.n_macroparticles_per_slice, counts)
    sums = torch.zeros(S, dtype=torch.float64, device='cuda')
    sums.index_add_(0, want[inside].long(), beam.x[inside].double())
    mean = torch.where(counts > 0, sums / counts.clamp(min=1).double(),
                       torch.zeros_like(sums))
    tol = 1e-12 if precision == 'fp64' else 1e-5   # FP32 slice sums
    assert float((mean - ss.mean_x).abs().max()) <= tol * float(
        mean.abs().max())


@pytest.mark.parametrize('name', ['linear_map', 'transverse_linear'])
def test_fixtures_without_transcendentals_are_bit_exact(lib, name):
    """Maps whose per-particle arithmetic is only +, -, *, / in the
    reference's order reproduce the reference bit for bit (the FP64 kernel
    rounds every operation separately, divisions included)."""
    import gpu_cases as G
    ref = load(os.path.join(GOLDEN, name + '.npz'))
    spec = json.loads(str(ref['spec']))
    beam = G.make_beam(spec['beam'], {k: ref['init_' + k] for k in COORDS})
    rec = G.run(spec, beam)
    t = spec['n_turns'] - 1
    for k in COORDS:
        np.testing.assert_array_equal(rec['t%d_%s' % (t, k)],
                                      ref['t%d_%s' % (t, k)], err_msg=k)


def test_division_by_host_constants_is_correctly_rounded(lib):
    """z / longfac in LinearMap runs the three-instruction division by a
    host reciprocal; compare 30 divisors x 131072 log-uniform dividends of
    both signs (3.9e6 quotients) with NumPy's IEEE division bit for bit."""
    import cases as C
    import gpu_cases as G
    from oracle import turn_loop as T
    rng = np.random.RandomState(42)
    n = 131072
    mag = 10.0 ** rng.uniform(-250, 250, n)
    z = mag * np.where(rng.rand(n) < 0.5, -1., 1.)
    dp = rng.normal(0, 1e-3, n)
    for i in range(30):
        Qs = 10.0 ** rng.uniform(-3, -0.5)
        alpha = C.GAMMA**-2 + 10.0 ** rng.uniform(-5, -1)
        coords = {k: np.zeros(n) for k in COORDS}
        coords['z'] = z
        coords['dp'] = dp
        beam = G.make_beam(C.beam_params(n, 0), coords)
        spec = dict(beam=C.beam_params(n, 0), n_turns=1,
                    elements=[C.linear_map(Q_s=Qs, alpha=alpha)])
        G.run(spec, beam)
        ob = T.Beam(coords, 1., beam.charge, beam.mass, beam.circumference,
                    beam.gamma)
        T.LinearMap([alpha], beam.circumference, Qs).track(ob)
        np.testing.assert_array_equal(beam.dp.cpu().numpy(), ob.dp,
                                      err_msg='divisor set %d' % i)
        np.testing.assert_array_equal(beam.z.cpu().numpy(), ob.z)


def test_thousand_slices_both_forms(lib):
    """C5's slicing (1000 slices, resonator + resistive wall): the shared
    memory plan falls back to fewer resident CTAs.  FP64 against the oracle
    at the usual bars.  FP32 against the oracle within 2e-4 of the RMS:
    with 20 particles per slice, a particle whose FP32 z rounds across a
    slice edge moves a few per cent of its slice's dipole moment, and the
    kicks of every trailing slice follow (measured 4e-5 after 8 turns)."""
    import cases as C
    import gpu_cases as G
    spec = dict(beam=C.beam_params(20000, 4), n_turns=8, elements=[
        C.smooth_transverse(chroma=[2., 2.],
                            amplitude=[1e-11, 1e-11, -5e-12]), C.rf(),
        C.wake(C.slicer(1000), C.resonator(),
               C.resistive_wall(n_turns_wake=5))])
    rec, ref = _oracle_vs_gpu(spec, 8, record_turns=(7,))
    compare(rec, ref, '1000 slices')
    from oracle import cases as OC
    c0 = OC.make_beam(spec['beam']).coords()
    b32 = G.make_beam(spec['beam'], c0, precision='fp32')
    r32 = G.run(spec, b32, n_turns=8, record_turns=(7,))
    for k in COORDS:
        assert rms_err(r32['t7_' + k], ref['t7_' + k]) <= 2e-4, k
