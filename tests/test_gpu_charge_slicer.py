"""UniformChargeSlicer on the GPU (order statistics without a sort).

The reference's own fixtures (charge_slicer, wake_charge_slicer) replay in
test_gpu_parity.py.  Here, at 2e5 macroparticles and 500 slices: the slice
index of every particle, the counts and z_bins equal the oracle's
argsort-based slicing bit for bit (FP64 form); in the FP32 form, every
particle whose index differs shares its z with another particle at a slice
edge (the documented tie case); and the slicer's random draws follow
Python's random module exactly as the reference's do.
"""
import random

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip('torch')


@pytest.fixture(scope='module')
def lib():
    from pyheadtail_gb300 import _native
    return _native.load()


@pytest.mark.parametrize('precision', ['fp64', 'fp32'])
@pytest.mark.parametrize('cuts,S', [((-0.5, 0.62), 500), (None, 333)])
def test_charge_slicing_matches_oracle(lib, precision, cuts, S):
    import cases as C
    import gpu_cases as G
    from oracle import cases as OC
    from oracle import turn_loop as T
    bp = C.beam_params(200000, 40)
    coords = OC.make_beam(bp).coords()
    if precision == 'fp32':
        coords = {k: v.astype(np.float32).astype(np.float64)
                  for k, v in coords.items()}
    sp = C.slicer(S, z_cuts=cuts, n_sigma_z=None if cuts else 3,
                  mode='uniform_charge')
    ob = OC.make_beam(bp, coords)
    random.seed(7)
    ref_bins, ref_idx = OC.make_slicer(sp).bins_and_index(ob)
    beam = G.make_beam(bp, coords, precision=precision)
    sl = G.make_slicer(sp)
    random.seed(7)
    ss = sl.slice(beam)
    idx = ss.slice_index_of_particle.cpu().numpy()
    z = coords['z']
    if cuts is None:
        # cuts from the bunch's mean and sigma: equal to the rounding of the
        # statistics (FP32 form: FP32 pair sums, ~1e-9), interior edges
        # (order statistics) exact
        tol = 1e-13 if precision == 'fp64' else 1e-8
        np.testing.assert_allclose(ss.z_bins[[0, -1]], ref_bins[[0, -1]],
                                   rtol=tol)
        np.testing.assert_array_equal(ss.z_bins[1:-1], ref_bins[1:-1])
    else:
        np.testing.assert_array_equal(ss.z_bins, ref_bins)
    bad = np.nonzero(idx != ref_idx)[0]
    if precision == 'fp64':
        assert len(bad) == 0, bad[:10]
        np.testing.assert_array_equal(
            ss.n_macroparticles_per_slice.cpu().numpy(),
            np.bincount(ref_idx[ref_idx >= 0], minlength=S))
    else:
        vals, counts = np.unique(z, return_counts=True)
        dup = set(vals[counts > 1])
        edges = set(ss._dslicer.edges.cpu().numpy().astype(np.float64))
        for i in bad:
            assert z[i] in dup and z[i] in edges, (i, z[i])
    # per-slice means over the slices the wake sees
    mx = ss.mean_x if hasattr(ss, 'mean_x') else None
    assert mx is None or mx.shape[0] == S
