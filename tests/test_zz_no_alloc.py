"""phk_slice_noalloc: the slicing pass whose partial sums live in a
library-owned device array, against the workspace entry points
phk_track + phk_slice_finalize on the same inputs, called through the C ABI,
and against an FP64 binning and summation on the host (the reference's
formula, int(floor((z - tail) / width)), particles/slicing.py:604-611).  The
large FP32 case has more partial columns than the scratch array holds (the
clamp to 128 columns, the kernel's tile loop covering the rest).

The file sorts last so that its GPU test also runs after every other test
has used the library in the same process; it passes alone as well."""
import ctypes

import numpy as np
import pytest
import torch

from pyheadtail_gb300 import _native as N
from pyheadtail_gb300._engine import DeviceSlicer

MAX_SLICES = 512      # capacity of the library-owned scratch array


def _coords(x, y, z, code, with_momenta):
    c = N.Coords()
    c.x, c.y, c.z = x.data_ptr(), y.data_ptr(), z.data_ptr()
    if with_momenta:
        c.xp, c.yp, c.dp = x.data_ptr(), y.data_ptr(), z.data_ptr()
    c.n = x.numel()
    c.dtype = code
    return c


def _with_workspace(L, sl, coords, stream):
    """phk_track (empty program, accumulation) + phk_slice_finalize with a
    torch-allocated partials workspace."""
    S = sl.n_slices
    grid = L.phk_track_grid(coords.n, coords.dtype, S)
    assert grid >= 1, N.last_error()
    partials = torch.empty(3 * S * grid, dtype=torch.float64, device='cuda')
    acc = N.Accum()
    acc.slicer = sl.struct
    acc.partials = partials.data_ptr()
    acc.partials_len = partials.numel()
    acc.grid = grid
    counts = torch.empty(S, dtype=torch.int32, device='cuda')
    mx = torch.empty(S, dtype=torch.float64, device='cuda')
    my = torch.empty(S, dtype=torch.float64, device='cuda')
    full = N.Coords()
    ctypes.memmove(ctypes.byref(full), ctypes.byref(coords),
                   ctypes.sizeof(N.Coords))
    full.xp, full.yp, full.dp = coords.x, coords.y, coords.z
    prog = N.Program()
    assert L.phk_track(ctypes.byref(prog), ctypes.byref(full), None,
                       ctypes.byref(acc), stream) == 0, N.last_error()
    assert L.phk_slice_finalize(ctypes.byref(acc), counts.data_ptr(),
                                mx.data_ptr(), my.data_ptr(), None,
                                stream) == 0, N.last_error()
    return counts, mx, my


def test_no_alloc_rejects_too_many_slices_before_any_cuda_call():
    L = N.load(build_if_missing=False)
    sl = N.Slicer()
    sl.n_slices = MAX_SLICES + 1
    sl.edges = 4096
    c = N.Coords()
    c.n = 10
    for f in ('x', 'y', 'z'):
        setattr(c, f, 8192)
    assert L.phk_slice_noalloc(ctypes.byref(sl), ctypes.byref(c), None, None,
                               None, None) == -2
    assert 'n_slices 513' in N.last_error()
    assert L.phk_slice_noalloc(None, ctypes.byref(c), None, None, None,
                               None) == -1
    sl.n_slices = 16
    c.x = 8196                       # not 8-byte aligned for FP64
    assert L.phk_slice_noalloc(ctypes.byref(sl), ctypes.byref(c), None, None,
                               None, None) == -3


def _host_reference(x, y, z, sl):
    """Counts and FP64 means per slice, binned on the host."""
    zh = z.double().cpu().numpy()
    idx = np.floor((zh - sl.tail) / sl.width)
    inside = (idx >= 0) & (idx < sl.n_slices)
    k = idx[inside].astype(np.int64)
    counts = np.bincount(k, minlength=sl.n_slices)
    out = [counts]
    for u in (x, y):
        sums = np.bincount(k, weights=u.double().cpu().numpy()[inside],
                           minlength=sl.n_slices)
        out.append(np.where(counts > 0, sums / np.maximum(counts, 1), 0.))
    return out


@pytest.mark.gpu
@pytest.mark.parametrize('code,n,S,with_momenta', [
    (0, 1_000_003, 500, False),
    (1, 1_000_003, 500, True),
    (0, 4099, MAX_SLICES, True),
    (1, 1, 7, False),
    (0, 10_000_000, 100, False),
    (1, 20_000_000, 100, True),
])
def test_no_alloc_matches_workspace_entry_point_twice(code, n, S,
                                                      with_momenta):
    L = N.load()
    dt = torch.float64 if code == 0 else torch.float32
    g = torch.Generator(device='cuda').manual_seed(1234 + n + S)
    x = torch.randn(n, generator=g, device='cuda', dtype=torch.float64)
    y = torch.randn(n, generator=g, device='cuda', dtype=torch.float64)
    z = 0.3 * torch.randn(n, generator=g, device='cuda', dtype=torch.float64)
    x, y, z = (1e-3 * x).to(dt), (1e-3 * y).to(dt), z.to(dt)
    sl = DeviceSlicer(-0.69, 0.69, S, code, 'cuda')
    coords = _coords(x, y, z, code, with_momenta)
    stream = torch.cuda.current_stream().cuda_stream
    if n >= 10_000_000 and code == 1:
        # more partial columns than the library-owned array holds (the
        # FP64 pass has fewer CTAs per SM: 74 clusters at this size)
        assert L.phk_track_grid(n, code, S) > 128
    ref_counts, ref_mx, ref_my = _with_workspace(L, sl, coords, stream)
    host_counts, host_mx, host_my = _host_reference(x, y, z, sl)
    np.testing.assert_array_equal(ref_counts.cpu().numpy(), host_counts)
    for call in range(2):
        counts = torch.full((S,), -7, dtype=torch.int32, device='cuda')
        mx = torch.full((S,), np.nan, dtype=torch.float64, device='cuda')
        my = torch.full((S,), np.nan, dtype=torch.float64, device='cuda')
        assert L.phk_slice_noalloc(ctypes.byref(sl.struct),
                                   ctypes.byref(coords), counts.data_ptr(),
                                   mx.data_ptr(), my.data_ptr(),
                                   stream) == 0, N.last_error()
        torch.cuda.synchronize()
        assert torch.equal(counts, ref_counts), call
        assert int(counts.sum()) <= n
        np.testing.assert_array_equal(counts.cpu().numpy(), host_counts)
        # FP64: both passes sum in FP64 over different column counts, the
        # host sequentially; bar: a sum of n terms in any order, relative to
        # the largest |u|.  FP32 coordinates: the per-slice sums are exact
        # fixed-point sums at a power-of-two scale per thread-block cluster
        # (the largest |u| of its first tiles maps to [2^26, 2^27)), so each
        # value rounds by at most 2^-27 of the largest |u|.
        for got, want, host, u in ((mx, ref_mx, host_mx, x),
                                   (my, ref_my, host_my, y)):
            got, want = got.cpu().numpy(), want.cpu().numpy()
            umax = float(u.abs().max()) if n else 0.
            if code == 0:
                bar = max(n, 1) * 2.0**-52 * umax
            else:
                bar = 2.0**-27 * umax * (1 + 1e-9) + max(n, 1) * 2.0**-52 * umax
            for other in (want, host):
                assert np.max(np.abs(got - other)) <= bar, (call, bar)
