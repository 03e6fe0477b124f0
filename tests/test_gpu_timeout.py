"""The bounded waits of the kernels, made to run out without any fault.

phk_set_wait_limit(0) makes every first-level wait of a kernel give up at
once while its bulk copies (or tensor-core MMAs) are genuinely in flight.
The kernel must then store PHK_DEV_TIMEOUT in its status word, wait for
what it has in flight with the default limit, free its tensor memory and
return; the context stays usable and the next launch, with the default
limit restored, computes the right result."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip('torch')


@pytest.fixture
def lib():
    from pyheadtail_gb300 import _native as N
    L = N.load()
    yield L
    L.phk_set_wait_limit(-1)


def _coords(n, seed):
    from pyheadtail_gb300 import _native as N
    g = torch.Generator(device='cuda').manual_seed(seed)
    t = {k: (torch.randn(n, generator=g, device='cuda') * s).float()
         for k, s in (('x', 1e-3), ('xp', 1e-5), ('y', 1e-3), ('yp', 1e-5),
                      ('z', 0.2), ('dp', 1e-3))}
    c = N.Coords()
    for k, v in t.items():
        setattr(c, k, v.data_ptr())
    c.n = n
    c.dtype = N.PHK_F32
    return t, c


def _program(status):
    from pyheadtail_gb300 import _native as N
    prog = N.Program()
    prog.n_ops = 1
    op = prog.op[0]
    op.kind = N.OP_TRANSVERSE
    f = np.zeros(64, dtype=np.float32)
    f[0:8] = [0.6, 40., -0.016, 0.6, 0.5, 45., -0.0166, 0.5]
    ctypes.memmove(ctypes.addressof(op.p), f.ctypes.data, 256)
    prog.status = status.data_ptr()
    return prog


def test_track_kernel_copy_wait_runs_out(lib):
    """FP32, 16-byte aligned: the fused pass streams through its TMA ring."""
    from pyheadtail_gb300 import _native as N
    from pyheadtail_gb300 import _engine as E
    n = 2_000_003
    t, c = _coords(n, 3)
    x0 = {k: v.clone() for k, v in t.items()}
    status = torch.zeros(1, dtype=torch.int32, device='cuda')
    prog = _program(status)
    lib.phk_set_wait_limit(0)
    assert lib.phk_track(ctypes.byref(prog), ctypes.byref(c), None, None,
                         E.stream_handle()) == 0
    torch.cuda.synchronize()
    assert int(status.item()) == N.PHK_DEV_TIMEOUT
    # default limit: the same map from the original coordinates completes
    lib.phk_set_wait_limit(-1)
    for k in t:
        t[k].copy_(x0[k])
    status.zero_()
    assert lib.phk_track(ctypes.byref(prog), ctypes.byref(c), None, None,
                         E.stream_handle()) == 0
    torch.cuda.synchronize()
    assert int(status.item()) == 0
    want = 0.6 * x0['x'].double() + 40. * x0['xp'].double()
    err = (t['x'].double() - want).abs().max().item()
    assert err <= 1e-6 * want.abs().max().item()


def test_tensor_core_wake_waits_run_out(lib):
    """The GEMM's waits for the MMAs that read a shared-memory stage give
    up; the kernel waits (bounded) for the MMAs in flight, frees its tensor
    memory, and the next call gives the FP64 convolution's kicks."""
    import sys, os
    sys.path.insert(0, os.path.dirname(__file__))
    import test_gpu_wake_tc as T
    from pyheadtail_gb300 import _native as N
    from pyheadtail_gb300 import _engine as E
    from pyheadtail_gb300.impedances.wakes import _TensorWake
    wf, times, ages, beta, moments, R = T._setup(500, 50, seed=5)
    nk = len(wf.wake_kicks)
    ref = torch.zeros(nk, 500, dtype=torch.float64, device='cuda')
    got = torch.zeros(nk, 500, dtype=torch.float32, device='cuda')
    ws = T._wake_set(wf, times, ages, beta, moments, R, 0, ref, N.PHK_F64)
    N.call('phk_wake', ctypes.byref(ws), E.stream_handle())
    ws = T._wake_set(wf, times, ages, beta, moments, R, 0, got, N.PHK_F32)
    tw = _TensorWake(moments.device)
    status = torch.zeros(1, dtype=torch.int32, device='cuda')
    tw.run(wf.wake_kicks, ws)            # expansion and first run
    tw.w.status = status.data_ptr()
    lib.phk_set_wait_limit(0)
    tw.run(wf.wake_kicks, ws)
    torch.cuda.synchronize()
    assert int(status.item()) == N.PHK_DEV_TIMEOUT
    lib.phk_set_wait_limit(-1)
    status.zero_()
    got.zero_()
    tw.run(wf.wake_kicks, ws)
    torch.cuda.synchronize()
    assert int(status.item()) == 0
    r, g = ref.cpu().numpy(), got.double().cpu().numpy()
    for k in range(nk):
        assert np.max(np.abs(g[k] - r[k])) <= 2e-4 * np.max(np.abs(r[k]))
