"""Particles.__add__ / __radd__ (merging beams, sum()) and extract_slices
(particles/particles.py:150-207, 264-305) on the GPU: coordinates and ids
concatenated exactly; one Particles per slice with the particles of that
slice in index order and its slice_info, the particles outside the cuts in
a last one as include_non_sliced asks."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip('torch')

COORDS = ('x', 'xp', 'y', 'yp', 'z', 'dp')


def _beam(n, seed, precision='fp64'):
    import cases as C
    import gpu_cases as G
    from oracle import cases as OC
    bp = C.beam_params(n, seed)
    coords = OC.make_beam(bp).coords()
    return G.make_beam(bp, coords, precision=precision), coords


def _np(t):
    return t.double().cpu().numpy()


def test_add_and_sum_merge_beams():
    b1, c1 = _beam(1000, 3)
    b2, c2 = _beam(777, 4)
    for m in (b1 + b2, sum([b1, b2])):
        assert m.macroparticlenumber == 1777
        for k in COORDS:
            np.testing.assert_array_equal(_np(getattr(m, k)),
                                          np.concatenate([c1[k], c2[k]]))
        np.testing.assert_array_equal(
            m.id.cpu().numpy(),
            np.concatenate([np.arange(1, 1001), np.arange(1, 778)]))
        x = np.concatenate([c1['x'], c2['x']])
        assert abs(m.mean_x() - np.mean(x)) <= 1e-12 * np.std(x)
    c = 0 + b1
    c.x = c.x * 2
    np.testing.assert_array_equal(_np(b1.x), c1['x'])


def test_extract_slices():
    import cases as C
    import gpu_cases as G
    b, c = _beam(5000, 5)
    S = 20
    sl = G.make_slicer(C.slicer(S))
    tail, head = C.Z_CUTS
    want = np.floor((c['z'] - tail) / ((head - tail) / float(S)))
    inside = (want >= 0) & (want < S)
    assert (~inside).any()
    parts = b.extract_slices(sl)
    assert len(parts) == S + 1
    ss = b.get_slices(sl)
    for i in range(S):
        sel = np.nonzero(want == i)[0]
        assert parts[i].macroparticlenumber == len(sel)
        np.testing.assert_array_equal(parts[i].id.cpu().numpy(), sel + 1)
        for k in COORDS:
            np.testing.assert_array_equal(_np(getattr(parts[i], k)),
                                          c[k][sel])
        info = parts[i].slice_info
        assert info['z_bin_left'] == ss.z_bins[i]
        assert info['z_bin_right'] == ss.z_bins[i + 1]
        assert info['z_bin_center'] == ss.z_centers[i]
    out = np.nonzero(~inside)[0]
    assert parts[-1].slice_info == 'unsliced'
    np.testing.assert_array_equal(parts[-1].id.cpu().numpy(), out + 1)
    assert len(b.extract_slices(sl, include_non_sliced='never')) == S
    assert len(b.extract_slices(sl, include_non_sliced='always')) == S + 1
    with pytest.raises(ValueError):
        b.extract_slices(sl, include_non_sliced='sometimes')


@pytest.mark.parametrize('mode', ['uniform_bin', 'uniform_charge'])
def test_compute_sliceset_kwargs(mode):
    """Slicer.compute_sliceset_kwargs gives the arguments of the SliceSet
    that slice() makes from the same state."""
    import cases as C
    import gpu_cases as G
    import random
    b, c = _beam(3000, 6)
    sl = G.make_slicer(C.slicer(30, mode=mode))
    # uniform-charge slicing hands the remainder particles to random
    # slices (the reference's random.sample): same seed for both
    random.seed(11)
    kw = sl.compute_sliceset_kwargs(b)
    random.seed(11)
    ss = sl.slice(b)
    assert set(kw) == {'z_bins', 'slice_index_of_particle', 'mode',
                       'n_macroparticles_per_slice'}
    assert kw['mode'] == ss.mode == mode
    np.testing.assert_array_equal(kw['z_bins'], ss.z_bins)
    assert torch.equal(kw['slice_index_of_particle'],
                       ss.slice_index_of_particle)
    assert torch.equal(kw['n_macroparticles_per_slice'],
                       ss.n_macroparticles_per_slice)
