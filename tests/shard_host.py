"""Host restatement of the compensated slice sums of a sharded bunch
(phk_slice_sums, phk_slice_merge in csrc/phk_kernels.cu), operation for
operation in IEEE double: the checker of the GPU kernels and of the
rank-ordered merge."""
import numpy as np


def two_sum(a, b):
    """Knuth's TwoSum, elementwise: s + e == a + b exactly."""
    s = a + b
    bb = s - a
    e = (a - (s - bb)) + (b - bb)
    return s, e


def combine(hi, lo, bh, bl):
    s, e = two_sum(hi, bh)
    return s, (lo + bl) + e


def fold_columns(P):
    """P: float64 [3, S, G] partial columns -> [2, 3, S] (high, low) pairs,
    in the kernel's order: lane l adds columns l, l + 32, ... in turn, then
    the lanes combine in the butterfly l ^ 16, ^ 8, ^ 4, ^ 2, ^ 1 and lane 0
    holds the result."""
    P = np.asarray(P, dtype=np.float64)
    q, S, G = P.shape
    hi = np.zeros((32, q, S))
    lo = np.zeros((32, q, S))
    for lane in range(32):
        for g in range(lane, G, 32):
            s, e = two_sum(hi[lane], P[:, :, g])
            hi[lane] = s
            lo[lane] = lo[lane] + e
    for o in (16, 8, 4, 2, 1):
        partner = np.arange(32) ^ o
        h2, l2 = combine(hi, lo, hi[partner], lo[partner])
        hi, lo = h2, l2
    return np.stack([hi[0], lo[0]])


def merge_pairs(pairs):
    """[R, 2, 3, S] pairs of R shards -> totals [3, S] (shard 0 first)."""
    pairs = np.asarray(pairs, dtype=np.float64)
    hi, lo = pairs[0, 0].copy(), pairs[0, 1].copy()
    for r in range(1, pairs.shape[0]):
        hi, lo = combine(hi, lo, pairs[r, 0], pairs[r, 1])
    return hi + lo


def finalize(totals):
    """Counts, means and wake moments from merged totals, as the kernel
    writes them."""
    n = totals[0].astype(np.int32)
    with np.errstate(invalid='ignore', divide='ignore'):
        mx = np.where(n > 0, totals[1] / np.maximum(n, 1), 0.0)
        my = np.where(n > 0, totals[2] / np.maximum(n, 1), 0.0)
    moments = np.stack([n.astype(np.float64), n * mx, n * my])
    return n, mx, my, moments
