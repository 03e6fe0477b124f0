"""Bunch statistics on the GPU (phk_bunch_stats behind Particles.mean_* ...
gamma_Twiss_*, and BunchMonitor).

* After a turn that ends with a WakeField (dipolar, quadrupolar and
  longitudinal kicks still pending on the device), all 26 statistics agree
  with the oracle's (which is bit-identical to the reference on the
  ``bunch_statistics`` fixture) to 1e-12, plain FP64 form, at 2e5
  macroparticles; the pending kicks are not applied to memory by the
  statistics.
* One pass per state: asking any number of statistics of one state launches
  one kernel; the coordinates and order asked for are remembered.
* Ragged sizes (n = 1 ... 100003), unaligned coordinate views (the scalar
  path), the cursor ring and a CUDA-graph replay of the statistics pass,
  and the FP32 form (Kahan FP32 first sums, FP32 pair sums, FP64 merge)
  against FP64 statistics of the same FP32 coordinates.
"""
import ctypes
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip('torch')

COORDS = ('x', 'xp', 'y', 'yp', 'z', 'dp')
GOLDEN = os.path.join(os.path.dirname(__file__), 'golden')


def _scale(ref_stats, name):
    v = abs(ref_stats[name])
    if name.startswith('mean_'):
        v = max(v, ref_stats['sigma_' + name[5:]])
    return v


def _oracle_stats(coords, gamma, p0, names):
    from oracle import turn_loop as T
    from scipy.constants import e, m_p
    b = T.Beam(coords, 1., e, m_p, 6911.5, gamma)
    b.p0 = p0
    return {n: float(getattr(b, n)()) for n in names}


@pytest.fixture(scope='module')
def lib():
    from pyheadtail_gb300 import _native
    return _native.load()


def test_all_statistics_with_pending_kicks_fp64(lib):
    import cases as C
    import gpu_cases as G
    from oracle import cases as OC
    from pyheadtail_gb300 import _native as N
    spec = dict(C.CASES['bunch_statistics'])
    spec['beam'] = C.beam_params(200000, 23, alpha_x=0.4, alpha_y=-0.3)
    ob = OC.make_beam(spec['beam'])
    coords = ob.coords()
    ref = OC.run(spec, ob, n_turns=2, record_turns=(1,))
    beam = G.make_beam(spec['beam'], coords)
    els = G.make_elements(spec, beam)
    for _ in range(2):
        for _, el in els:
            el.track(beam)
    assert beam._engine.kick is not None          # kicks still pending
    n0 = N.launch_count()
    got = {n: getattr(beam, n)() for n in C.BUNCH_STATS}
    launched = N.launch_count() - n0
    assert beam._engine.kick is not None          # and still pending
    refs = {n: float(ref['t1_bs_' + n]) for n in C.BUNCH_STATS}
    for n in C.BUNCH_STATS:
        assert abs(got[n] - refs[n]) <= 1e-12 * _scale(refs, n), \
            (n, got[n], refs[n])
    # the first state learns what is asked (the union of coordinates and
    # the highest order grows with each miss: six means, then order 2), and
    # every later state needs one pass for all 26
    assert launched <= 7, launched
    for _, el in els:
        el.track(beam)
    n0 = N.launch_count()
    for n in C.BUNCH_STATS:
        getattr(beam, n)()
    assert N.launch_count() - n0 == 1


def _direct(code, coords_np, order=2, mask=0x3f, offset=0, capacity=1,
            cursor=None, records=None):
    """phk_bunch_stats through the C ABI on views starting at `offset`."""
    from pyheadtail_gb300 import _native as N
    dt = torch.float64 if code == N.PHK_F64 else torch.float32
    n = len(coords_np['x'])
    ts = {}
    for q in COORDS:
        t = torch.zeros(n + offset, dtype=dt, device='cuda')
        t[offset:] = torch.from_numpy(np.asarray(coords_np[q])).to(dt)
        ts[q] = t
    c = N.Coords()
    for q in COORDS:
        setattr(c, q, ts[q][offset:].data_ptr())
    c.n, c.dtype = n, code
    grid = N.call('phk_bunch_stats_grid', n, code)
    part = torch.empty(grid * N.PHK_STATS_LEN, dtype=torch.float64,
                       device='cuda')
    ticket = torch.zeros(1, dtype=torch.int32, device='cuda')
    if records is None:
        records = torch.full((capacity * N.PHK_STATS_LEN,), -7.,
                             dtype=torch.float64, device='cuda')
    st = N.Stats()
    st.order, st.capacity, st.grid, st.mask = order, capacity, grid, mask
    st.records, st.partials = records.data_ptr(), part.data_ptr()
    st.ticket = ticket.data_ptr()
    st.cursor = 0 if cursor is None else cursor.data_ptr()
    N.call('phk_bunch_stats', ctypes.byref(c), None, ctypes.byref(st),
           ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    torch.cuda.synchronize()
    assert int(ticket.item()) == 0
    return records.cpu().numpy(), ts, (c, st, part, ticket)


@pytest.mark.parametrize('n', [1, 2, 3, 257, 513, 1000, 100003])
@pytest.mark.parametrize('offset', [0, 1])
def test_ragged_and_unaligned_fp64(lib, n, offset):
    from pyheadtail_gb300.particles import statistics as S
    rng = np.random.RandomState(n)
    c = {q: rng.normal(loc=0.3, scale=1e-3, size=n) for q in COORDS}
    r, _, _ = _direct(0, c, offset=offset)
    rec = S.StatsRecord(r)
    assert rec.n == n
    for q in COORDS:
        assert r[1 + COORDS.index(q)] == c[q][0]     # the reference's shift
        assert abs(rec.mean(q) - np.mean(c[q])) <= 1e-12 * 1e-3
    if n > 1:
        from oracle import turn_loop as T
        for qa, qb in S.USED_PAIRS:
            want = T.cov_shifted(c[qa], c[qb])
            assert abs(rec.cov(qa, qb) - want) <= 1e-12 * 1e-6, (qa, qb)
        # cross-plane pairs are not summed
        assert r[13 + 2] == 0.0 and r[13 + 6 + 1] == 0.0


def test_order_one_and_mask(lib):
    rng = np.random.RandomState(3)
    c = {q: rng.normal(size=5000) for q in COORDS}
    for offset in (0, 1):            # the compact and the general kernel
        r, _, _ = _direct(0, c, order=1, mask=(1 << 0) | (1 << 4),
                          offset=offset)
        assert r[0] == 5000
        assert np.all(r[1:7] == 0)           # order 1: plain sums
        assert abs(r[7] - np.sum(c['x'])) <= 1e-11
        assert abs(r[11] - np.sum(c['z'])) <= 1e-11
        assert r[8] == 0 and r[9] == 0 and r[10] == 0 and r[12] == 0
        assert np.all(r[13:] == 0)
    r32, _, _ = _direct(1, c, order=1, mask=0x3f)
    for i, q in enumerate(COORDS):
        assert abs(r32[7 + i] - np.sum(c[q].astype(np.float32).astype(
            np.float64))) <= 1e-4, q


def test_cursor_ring_and_graph_replay(lib):
    from pyheadtail_gb300 import _native as N
    rng = np.random.RandomState(4)
    c = {q: rng.normal(size=20000) for q in COORDS}
    cursor = torch.zeros(1, dtype=torch.int64, device='cuda')
    records = torch.zeros(3 * N.PHK_STATS_LEN, dtype=torch.float64,
                          device='cuda')
    r, ts, (cs, st, part, ticket) = _direct(0, c, capacity=3, cursor=cursor,
                                            records=records)
    assert int(cursor.item()) == 1
    first = r[:N.PHK_STATS_LEN].copy()
    assert np.all(r[N.PHK_STATS_LEN:] == 0)
    # capture one pass into a graph; each replay appends to the next slot
    g = torch.cuda.CUDAGraph()
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        with torch.cuda.graph(g, stream=s):
            N.call('phk_bunch_stats', ctypes.byref(cs), None,
                   ctypes.byref(st), ctypes.c_void_p(s.cuda_stream))
    torch.cuda.current_stream().wait_stream(s)
    torch.cuda.synchronize()
    # capture ran nothing: the cursor is where the eager call left it
    assert int(cursor.item()) == 1
    for k in range(4):
        ts['x'].add_(1.0)
        g.replay()
    torch.cuda.synchronize()
    assert int(cursor.item()) == 5
    assert int(ticket.item()) == 0
    rows = records.view(3, N.PHK_STATS_LEN).cpu().numpy()
    # replays 1..4 went to slots 1, 2, 0, 1; the last one saw x + 4
    assert abs(rows[1][1] - (c['x'][0] + 4.0)) <= 1e-15 * 8
    np.testing.assert_array_equal(rows[1][2:7], first[2:7])
    np.testing.assert_allclose(rows[1][7:], first[7:], rtol=1e-12, atol=1e-9)


def test_fp32_form_against_fp64_of_same_coordinates(lib):
    from pyheadtail_gb300.particles import statistics as S
    from oracle import turn_loop as T
    rng = np.random.RandomState(8)
    n = 1000003
    c = {q: rng.normal(loc=2e-4, scale=1e-3, size=n).astype(np.float32)
         for q in COORDS}
    r, _, _ = _direct(1, c)
    rec = S.StatsRecord(r)
    c64 = {q: c[q].astype(np.float64) for q in COORDS}
    for q in COORDS:
        sig = np.std(c64[q])
        assert abs(rec.mean(q) - np.mean(c64[q])) <= 1e-7 * sig, q
        assert abs(rec.std(q) - T.std(c64[q])) <= 1e-6 * sig, q
    e_got = rec.emittance('x', 'xp', 'dp')
    e_want = T.emittance(c64['x'], c64['xp'], c64['dp'])
    assert abs(e_got - e_want) <= 1e-5 * e_want


def test_fp32_beam_statistics_with_pending_kicks(lib):
    """FP32 form after a wake turn: statistics of the state with the kicks
    pending equal (to FP32-sum accuracy) the FP64 statistics of the FP32
    coordinates after the kicks are applied to memory."""
    import cases as C
    import gpu_cases as G
    from oracle import cases as OC
    spec = dict(C.CASES['bunch_statistics'])
    spec['beam'] = C.beam_params(300000, 23, alpha_x=0.4, alpha_y=-0.3)
    coords = OC.make_beam(spec['beam']).coords()
    beam = G.make_beam(spec['beam'], coords, precision='fp32')
    for _, el in G.make_elements(spec, beam):
        el.track(beam)
    assert beam._engine.kick is not None
    got = {n: getattr(beam, n)() for n in C.BUNCH_STATS}
    c = beam.coords_numpy()           # applies the kicks in memory
    ref = _oracle_stats(c, beam.gamma, beam.p0, C.BUNCH_STATS)
    for n in C.BUNCH_STATS:
        tol = 1e-6 if n.startswith(('mean_', 'sigma_')) else 1e-4
        assert abs(got[n] - ref[n]) <= tol * _scale(ref, n), (n, got[n], ref[n])


def test_bunch_monitor_on_gpu(lib, tmp_path):
    import cases as C
    import gpu_cases as G
    from oracle import cases as OC
    from pyheadtail_gb300.monitors.monitors import BunchMonitor
    spec = dict(C.CASES['wake_resonator'])
    spec['beam'] = C.beam_params(50000, 19)
    beam = G.make_beam(spec['beam'], OC.make_beam(spec['beam']).coords())
    els = G.make_elements(spec, beam)
    stats = ['mean_x', 'mean_xp', 'sigma_x', 'epsn_x', 'epsn_z',
             'macroparticlenumber']
    fn = str(tmp_path / 'mon')
    mon = BunchMonitor(fn, 7, write_buffer_every=3, buffer_size=3,
                       stats_to_store=stats)
    direct = {s: [] for s in stats}
    for _ in range(7):
        for _, el in els:
            el.track(beam)
        mon.dump(beam)
        for s in stats:
            v = getattr(beam, s)
            direct[s].append(v() if callable(v) else v)
    out = (np.load(fn + '.npz') if os.path.exists(fn + '.npz') else None)
    if out is None:
        pytest.skip('h5py output')
    for s in stats:
        np.testing.assert_allclose(out[s], direct[s], rtol=1e-14, err_msg=s)


def test_slice_and_particle_monitors_on_gpu(lib, tmp_path):
    """SliceMonitor and ParticleMonitor on a GPU bunch after a wake turn:
    the file holds what the slice set and the bunch report directly."""
    import os
    import cases as C
    import gpu_cases as G
    from oracle import cases as OC
    from pyheadtail_gb300.monitors.monitors import (ParticleMonitor,
                                                    SliceMonitor)
    spec = dict(C.CASES['wake_resonator'])
    spec['beam'] = C.beam_params(30000, 19)
    beam = G.make_beam(spec['beam'], OC.make_beam(spec['beam']).coords())
    els = G.make_elements(spec, beam)
    sl = G.make_slicer(C.slicer(20))
    fn = str(tmp_path / 'sm')
    sm = SliceMonitor(fn, 3, sl, write_buffer_every=2, buffer_size=2)
    pm = ParticleMonitor(str(tmp_path / 'pm'), stride=7)
    counts, mean_x = [], []
    for _ in range(3):
        for _, el in els:
            el.track(beam)
        sm.dump(beam)
        pm.dump(beam)
        ss = beam.get_slices(sl, statistics=True)
        counts.append(ss.n_macroparticles_per_slice.cpu().numpy())
        mean_x.append(beam.mean_x())
    if not os.path.exists(fn + '.npz'):
        pytest.skip('h5py output')
    with np.load(fn + '.npz') as f:
        np.testing.assert_array_equal(f['Slices/n_macroparticles_per_slice'],
                                      np.array(counts).T)
        np.testing.assert_allclose(f['Bunch/mean_x'], mean_x, rtol=0,
                                   atol=1e-12 * beam.sigma_x())
    with np.load(str(tmp_path / 'pm') + '.Step#2.npz') as f:
        np.testing.assert_array_equal(f['x'], beam.x.cpu().numpy()[::7])
