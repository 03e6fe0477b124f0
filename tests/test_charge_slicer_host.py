"""UniformChargeSlicer's host tables (no GPU): with the three device steps
emulated in NumPy (histogram on the kernels' bin formula, gather, select),
the order statistics, z_bins and slice edges reproduce the reference's
argsort-based slicing (the oracle, pinned on the charge_slicer fixture)."""
import random

import numpy as np
import pytest

from oracle import turn_loop as T

pytest.importorskip('torch')

from pyheadtail_gb300.particles import slicing as SL  # noqa: E402


def emulate(z, tail, head, S, code, seed):
    n = len(z)
    K = SL.charge_bins_for(n)
    scale = K / (head - tail)
    zz = z.astype(np.float64)
    inside = (zz >= tail) & (zz < head)
    b = np.clip(((zz[inside] - tail) * scale).astype(np.int64), 0, K - 1)
    h = np.bincount(b, minlength=K)
    n_cut_tail = int(np.sum(zz < tail))
    n_cut_head = n - int(np.sum(zz < head))
    random.seed(seed)
    per_slice, ranks = SL.charge_ranks(n, n_cut_tail, n_cut_head, S)
    tab = SL.charge_segments(h, ranks)
    vals = []
    zin = zz[inside]
    for s, r in zip(tab['tgt_seg'], tab['tgt_rank']):
        bin_ = np.nonzero(tab['seg_of_bin'] == s)[0][0]
        seg = np.sort(zin[b == bin_])
        assert len(seg) == tab['seg_count'][s]
        vals.append(seg[r])
    z_bins, edges = SL.charge_bins_and_edges(np.array(vals), tail, head, S,
                                             code)
    return per_slice, z_bins, edges


@pytest.mark.parametrize('n,S,cuts', [(1203, 37, (-0.69, 0.69)),
                                      (50000, 500, (-0.5, 0.6)),
                                      (999, 16, (-0.2, 0.35))])
@pytest.mark.parametrize('code', [0, 1])
def test_tables_reproduce_argsort_slicing(n, S, cuts, code):
    rng = np.random.RandomState(n)
    z = rng.normal(0, 0.23, n)
    if code == 1:
        z = z.astype(np.float32).astype(np.float64)
    tail, head = cuts
    per_slice, z_bins, edges = emulate(z, tail, head, S, code, seed=S)
    # the oracle's argsort slicing with the same random draws
    beam = T.Beam({k: (z if k == 'z' else np.zeros(n))
                   for k in T.Beam.COORDS}, 1., 1., 1., 1., 27.7)
    sl = T.UniformChargeSlicer(S, z_cuts=cuts)
    random.seed(S)
    ref_bins, ref_idx = sl.bins_and_index(beam)
    np.testing.assert_array_equal(z_bins, ref_bins)
    # binning on the edges gives the reference's indices, except for
    # particles sharing their z with another particle at a slice edge (the
    # reference's choice among equal keys is its sort's)
    zd = z.astype(edges.dtype)
    k = np.searchsorted(edges, zd, side='right') - 1
    inside = (zd >= edges[0]) & (zd < edges[-1])
    idx = np.where(inside, k, -1)
    bad = np.nonzero(idx != ref_idx)[0]
    vals, counts = np.unique(zd, return_counts=True)
    dup = set(vals[counts > 1])
    for i in bad:
        assert zd[i] in dup and zd[i] in set(edges), (i, zd[i])
    if code == 0:
        assert len(bad) == 0
    if len(bad) == 0:
        np.testing.assert_array_equal(
            np.bincount(idx[idx >= 0], minlength=S), per_slice)
