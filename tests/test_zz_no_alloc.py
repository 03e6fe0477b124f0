"""phk_slice_noalloc: the slicing pass whose partial sums live in a
library-owned device array, against the workspace entry points
phk_track + phk_slice_finalize on the same inputs, called through the C ABI.

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


@pytest.mark.gpu
@pytest.mark.parametrize('code,n,S,with_momenta', [
    (0, 1_000_003, 500, False),
    (1, 1_000_003, 500, True),
    (0, 4099, MAX_SLICES, True),
    (1, 1, 7, False),
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
    ref_counts, ref_mx, ref_my = _with_workspace(L, sl, coords, stream)
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
        # FP64: the same kernel with the same column count sums in a fixed
        # order, so 1e-12 relative is a loose bar.  FP32 coordinates: with
        # many slices the CTAs share one histogram and add with shared-memory
        # float atomics, whose order varies from launch to launch; the bar
        # is 1e-7 of the coordinate RMS.
        for got, want, u in ((mx, ref_mx, x), (my, ref_my, y)):
            got, want = got.cpu().numpy(), want.cpu().numpy()
            if code == 0:
                np.testing.assert_allclose(got, want, rtol=1e-12, atol=0,
                                           equal_nan=True)
            else:
                rms = float(u.double().pow(2).mean().sqrt())
                np.testing.assert_allclose(got, want, rtol=0,
                                           atol=1e-7 * rms, equal_nan=True)
