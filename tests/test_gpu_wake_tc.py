"""Tensor-core wake (phk_wake_tc_*: Toeplitz GEMM on tcgen05, BF16x3 split
products, FP32 accumulation) against the FP64 SIMT convolution phk_wake on
the same sampled wake tables and moment ring.

Tolerance: each operand is split into two bfloat16 parts, which keeps it to
~4e-6 relative; products are exact in the tensor cores and summed in FP32
over up to 51 * 1000 terms, whose signs alternate for the resonator.  The
kicks must agree with the FP64 result to 2e-4 of the largest kick of the
plane (measured: a few 1e-6)."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip('torch')


@pytest.fixture(scope='module')
def lib():
    from pyheadtail_gb300 import _native as N
    return N.load()


def _setup(S, rw_turns, seed):
    from scipy.constants import c
    from pyheadtail_gb300.general.printers import SilentPrinter
    from pyheadtail_gb300.impedances import wakes as W
    from pyheadtail_gb300.particles.slicing import UniformBinSlicer
    sl = UniformBinSlicer(S, z_cuts=(-0.69, 0.69), warningprinter=SilentPrinter())
    sources = [W.CircularResonator(10e6, 1e9, 1.)]
    if rw_turns:
        sources.append(W.CircularResistiveWall(0.02, 6911.5, 5.8e7, 1e-12,
                                               n_turns_wake=rw_turns))
    wf = W.WakeField(sl, *sources)
    R = max(1, rw_turns)
    gamma = 27.7
    beta = np.sqrt(1 - gamma**-2)
    z_bins = sl.z_bins(-0.69, 0.69)
    times = sl.times(z_bins, beta)
    ages, a = [], 0.
    for _ in range(R):
        ages.append(a)
        a += 6911.5 / (beta * c)
    rng = np.random.default_rng(seed)
    zc = 0.5 * (z_bins[1:] + z_bins[:-1])
    counts = np.round(2e4 * np.exp(-0.5 * (zc / 0.23)**2))
    mom = np.zeros((R, 3, S))
    for r in range(R):
        mom[r, 0] = counts
        mom[r, 1] = counts * rng.normal(0, 1e-4, S)
        mom[r, 2] = counts * rng.normal(0, 1e-4, S)
    moments = torch.from_numpy(mom).cuda()
    return wf, times, ages, beta, moments, R


def _wake_set(wf, times, ages, beta, moments, R, head, out, code):
    from pyheadtail_gb300 import _native as N
    from pyheadtail_gb300.impedances.wake_kicks import _SOURCE
    S = len(times)
    ws = N.WakeSet()
    ws.n_slices, ws.ring_len, ws.head = S, R, head
    ws.n_kicks = len(wf.wake_kicks)
    ws.out_dtype = code
    ws.moments = moments.data_ptr()
    for k, kick in enumerate(wf.wake_kicks):
        st = ws.kick[k]
        st.n_lags = kick._sync_tables([times] * len(ages), ages,
                                      [beta] * len(ages), S, moments.device)
        st.source = _SOURCE[kick.moment]
        st.dense = 0
        st.factor = -1.7e-11 * (k + 1)
        st.table = kick._table.data_ptr()
        st.out = out[k].data_ptr()
    return ws


@pytest.mark.parametrize('S,rw_turns', [(100, 0), (128, 3), (500, 50),
                                        (1000, 50)])
def test_tensor_wake_matches_fp64_convolution(lib, S, rw_turns):
    from pyheadtail_gb300 import _native as N
    from pyheadtail_gb300 import _engine as E
    from pyheadtail_gb300.impedances.wakes import _TensorWake
    wf, times, ages, beta, moments, R = _setup(S, rw_turns, seed=S + rw_turns)
    nk = len(wf.wake_kicks)
    for head in sorted({0, R - 1, R // 2}):
        ref = torch.zeros(nk, S, dtype=torch.float64, device='cuda')
        got = torch.zeros(nk, S, dtype=torch.float32, device='cuda')
        ws = _wake_set(wf, times, ages, beta, moments, R, head, ref, N.PHK_F64)
        N.call('phk_wake', ctypes.byref(ws), E.stream_handle())
        ws = _wake_set(wf, times, ages, beta, moments, R, head, got, N.PHK_F32)
        tw = _TensorWake(moments.device)
        tw.run(wf.wake_kicks, ws)
        torch.cuda.synchronize()
        # x and y dipole kicks of each circular source share a table group
        assert tw.w.n_groups == (2 if rw_turns else 1)
        r, g = ref.cpu().numpy(), got.double().cpu().numpy()
        for k in range(nk):
            scale = np.max(np.abs(r[k]))
            assert scale > 0
            err = np.max(np.abs(g[k] - r[k])) / scale
            assert err <= 2e-4, (S, rw_turns, head, k, err)


def test_fp32_wakefield_uses_the_tensor_path(lib):
    """A FP32 WakeField with a multi-turn wake and fixed cuts launches
    phk_wake_tc_run (single-turn wakes stay on phk_wake), and its
    kicks track the FP64 WakeField's to the tolerance above."""
    import cases as C
    import gpu_cases as G
    from oracle import cases as OC
    from pyheadtail_gb300 import _native as N
    spec = dict(beam=C.beam_params(20000, 7), n_turns=6, elements=[
        C.smooth_transverse(), C.rf(),
        C.wake(C.slicer(200), C.resonator(),
               C.resistive_wall(n_turns_wake=4))])
    coords = OC.make_beam(spec['beam']).coords()
    calls = []
    N.RECORDERS.append(lambda name, args: calls.append(name))
    try:
        beams = {}
        for prec in ('fp64', 'fp32'):
            b = G.make_beam(spec['beam'], coords, precision=prec)
            els = [el for _, el in G.make_elements(spec, b)]
            for _ in range(spec['n_turns']):
                for el in els:
                    el.track(b)
            beams[prec] = (b, els)
    finally:
        N.RECORDERS.pop()
    assert 'phk_wake_tc_run' in calls and 'phk_wake' in calls
    k64 = beams['fp64'][1][-1]._state.kick_out.cpu().numpy()
    k32 = beams['fp32'][1][-1]._state.kick_out.double().cpu().numpy()
    for k in range(k64.shape[0]):
        scale = np.max(np.abs(k64[k]))
        # different FP32 vs FP64 trajectories over 6 turns dominate here
        assert np.max(np.abs(k32[k] - k64[k])) <= 1e-2 * scale
