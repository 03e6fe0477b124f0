"""SliceSet's analysis methods on the host (no GPU), against the
reference's own values (tests/golden/sliceset/analysis.npz, made by
make_golden_sliceset.py running PyHEADTAIL): smoothing_sigma,
particle_indices_by_slice, pidx_begin / pidx_end,
particles_within_cuts_slice, lambda_bins, lambda_prime_bins, lambda_z,
lambda_prime_z, and ModeIsUniformCharge for uniform-charge slicing.  The
SliceSet is given the reference's slicing directly (CPU tensors), so the
methods are compared on identical inputs: index arrays bit for bit, the
line densities to 1e-13 (scipy's Gaussian filter rounds differently on
x86 and Arm builds, by ~5e-16; on the machine that made the fixture they
agree bit for bit)."""
import os

import numpy as np
import pytest

torch = pytest.importorskip('torch')

from pyheadtail_gb300.particles import slicing as S  # noqa: E402

GOLDEN = os.path.join(os.path.dirname(__file__), 'golden')


class _Engine(object):
    z_version = 0


class _Beam(object):
    _engine = _Engine()


def _sliceset(g, tag):
    p = tag + '_'
    ss = S.SliceSet(g[p + 'z_bins'], str(g[p + 'mode']), None, _Beam(),
                    torch.from_numpy(g[p + 'counts']),
                    beam_parameters=dict(
                        charge_per_mp=float(g[p + 'charge_per_mp']),
                        is_sorted=False))
    ss._slice_index_of_particle = torch.from_numpy(g[p + 'idx'])
    return ss


def _close(got, want):
    np.testing.assert_allclose(got, want, rtol=1e-13,
                               atol=1e-13 * np.max(np.abs(want)))


@pytest.fixture(scope='module')
def golden():
    with np.load(os.path.join(GOLDEN, 'sliceset', 'analysis.npz')) as f:
        return {k: f[k] for k in f.files}


@pytest.mark.parametrize('tag', ['bin', 'charge'])
def test_sliceset_analysis_matches_reference(golden, tag):
    g, p = golden, tag + '_'
    ss = _sliceset(g, tag)
    assert ss.smoothing_sigma == g[p + 'smoothing_sigma']
    np.testing.assert_array_equal(ss.particle_indices_by_slice.numpy(),
                                  g[p + 'by_slice'])
    assert ss.pidx_begin == g[p + 'pidx_begin']
    assert ss.pidx_end == g[p + 'pidx_end']
    np.testing.assert_array_equal(
        np.asarray(ss.particles_within_cuts_slice), g[p + 'within'])
    _close(ss.lambda_bins(), g[p + 'lambda_bins'])
    _close(ss.lambda_bins(sigma=3., smoothen=False), g[p + 'lambda_bins_raw'])
    _close(ss.lambda_z(), g[p + 'lambda_z'])
    _close(ss.lambda_z(g['zq']), g[p + 'lambda_zq'])
    if p + 'lambda_prime_raises' in g:
        with pytest.raises(S.ModeIsUniformCharge):
            ss.lambda_prime_bins()
    else:
        _close(ss.lambda_prime_bins(), g[p + 'lambda_prime_bins'])
        _close(ss.lambda_prime_bins(sigma=2., smoothen_before=False),
               g[p + 'lambda_prime_bins_s2'])
        _close(ss.lambda_prime_z(g['zq']), g[p + 'lambda_prime_zq'])


def test_particle_indices_of_slice_agree_with_by_slice(golden):
    ss = _sliceset(golden, 'bin')
    pos = ss.slice_positions.numpy()
    by = ss.particle_indices_by_slice.numpy()
    for k in (0, 7, 31, ss.n_slices - 1):
        np.testing.assert_array_equal(ss.particle_indices_of_slice(k).numpy(),
                                      by[pos[k]:pos[k + 1]])


def test_update_slices_is_gone():
    sl = S.UniformBinSlicer(10, z_cuts=(-1., 1.))
    with pytest.raises(RuntimeError, match='update_slices'):
        sl.update_slices(None)
