"""CPU checks of the native boundary and of the host logic (no GPU calls).

* libphk.so builds for sm_103a, loads, and exports every entry point that
  include/pyheadtail_gb300.h declares;
* the ctypes structures have the C layout (sizes and offsets);
* the exact slice-edge tables reproduce int32(floor((z - tail)/width)) for
  every z, in FP64 and for FP32 coordinates, for both signs of the width.
"""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, 'include', 'pyheadtail_gb300.h')


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r'/\*.*?\*/', '', src, flags=re.S)
    return sorted(set(re.findall(r'\bint(?:64_t)?\s+(phk_\w+)\s*\(', src)))


@pytest.fixture(scope='module')
def lib():
    from pyheadtail_gb300 import _build
    path = _build.build()
    return ctypes.CDLL(path)


def test_library_exports_every_declared_entry_point(lib):
    names = declared_functions()
    assert len(names) >= 8
    for n in names:
        assert hasattr(lib, n), n
    from pyheadtail_gb300 import _native
    assert set(names) <= set(_native.SIGNATURES)


def test_abi_version(lib):
    lib.phk_abi_version.restype = ctypes.c_int
    assert lib.phk_abi_version() == 1


def test_host_validation_without_gpu(lib):
    """Argument errors are caught on the host before any CUDA call."""
    from pyheadtail_gb300 import _native as N
    L = N.load(build_if_missing=False)
    prog = N.Program()
    prog.n_ops = 99
    coords = N.Coords()
    assert L.phk_track(ctypes.byref(prog), ctypes.byref(coords), None, None,
                       None) == -2
    assert 'n_ops' in N.last_error()
    prog.n_ops = 0
    coords.n = -5
    assert L.phk_track(ctypes.byref(prog), ctypes.byref(coords), None, None,
                       None) == -2
    coords.n = 10
    coords.dtype = 7
    assert L.phk_track(ctypes.byref(prog), ctypes.byref(coords), None, None,
                       None) == -4
    coords.dtype = 0
    assert L.phk_track(ctypes.byref(prog), ctypes.byref(coords), None, None,
                       None) == -1          # NULL coordinate pointers
    for i, f in enumerate(('x', 'xp', 'y', 'yp', 'z', 'dp')):
        setattr(coords, f, 4096 * (i + 1) + 4)   # 4-byte aligned only
    assert L.phk_track(ctypes.byref(prog), ctypes.byref(coords), None, None,
                       None) == -3
    ws = N.WakeSet()
    ws.n_slices = 0
    assert L.phk_wake(ctypes.byref(ws), None) == -2
    acc = N.Accum()
    acc.slicer.n_slices = 10
    acc.slicer.edges = 4096
    acc.partials = 8192
    acc.grid = 4
    acc.partials_len = 100
    for i, f in enumerate(('x', 'xp', 'y', 'yp', 'z', 'dp')):
        setattr(coords, f, 4096 * (i + 1))
    assert L.phk_track(ctypes.byref(prog), ctypes.byref(coords), None,
                       ctypes.byref(acc), None) == -6
    assert 'partials' in N.last_error()


def test_struct_layout_matches_header():
    from pyheadtail_gb300 import _native as N
    assert ctypes.sizeof(N.Coords) == 64
    assert ctypes.sizeof(N.Slicer) == 48
    assert ctypes.sizeof(N.Op) == 24 + 32 * 8
    assert ctypes.sizeof(N.Detuner) == 24 + 16 * 8
    assert ctypes.sizeof(N.Program) == 8 + 12 * 280 + 6 * 152 + 8
    assert N.KickSet.kick.offset == 120
    assert ctypes.sizeof(N.KickSet) == 184
    assert ctypes.sizeof(N.Accum) == 80
    assert ctypes.sizeof(N.WakeKick) == 40
    assert N.WakeSet.kick.offset == 32
    assert ctypes.sizeof(N.Stats) == 56
    assert N.Stats.means.offset == 40


def test_stats_and_damper_validation_without_gpu(lib):
    """phk_bunch_stats and the damper op reject bad arguments on the host."""
    from pyheadtail_gb300 import _native as N
    L = N.load(build_if_missing=False)
    c = N.Coords()
    for i, f in enumerate(('x', 'xp', 'y', 'yp', 'z', 'dp')):
        setattr(c, f, 4096 * (i + 1))
    c.n, c.dtype = 100, 0
    st = N.Stats()
    st.order, st.capacity, st.grid = 3, 1, 1
    st.records, st.partials, st.ticket = 8192, 16384, 32768
    assert L.phk_bunch_stats(ctypes.byref(c), None, ctypes.byref(st),
                             None) == -4
    st.order = 2
    st.capacity = 0
    assert L.phk_bunch_stats(ctypes.byref(c), None, ctypes.byref(st),
                             None) == -2
    st.capacity = 1
    st.mask = 0x40
    assert L.phk_bunch_stats(ctypes.byref(c), None, ctypes.byref(st),
                             None) == -4
    st.mask = 0
    st.ticket = 0
    assert L.phk_bunch_stats(ctypes.byref(c), None, ctypes.byref(st),
                             None) == -1
    st.ticket = 32768
    st.means = 12
    assert L.phk_bunch_stats(ctypes.byref(c), None, ctypes.byref(st),
                             None) == -3
    assert L.phk_bunch_stats_grid(-1, 0) == -2
    prog = N.Program()
    prog.n_ops = 1
    prog.op[0].kind = N.OP_DAMPER
    assert L.phk_track(ctypes.byref(prog), ctypes.byref(c), None, None,
                       None) == -4           # no means pointer
    assert 'damper' in N.last_error()


@pytest.mark.parametrize('code', [0, 1])
@pytest.mark.parametrize('cuts,S', [((-0.69, 0.69), 50), ((-0.31, 0.05), 7),
                                    ((0.2, -0.2), 13), ((-3e-3, 1e-2), 500),
                                    ((-1.1, 1.3), 1000)])
def test_exact_edges_reproduce_reference_index(code, cuts, S):
    from pyheadtail_gb300 import _engine as E
    tail, head = cuts
    width = (head - tail) / float(S)
    e, neg = E.exact_edges(tail, width, S, code)
    dt = np.float64 if code == 0 else np.float32
    rng = np.random.RandomState(S)
    span = abs(head - tail)
    z = (rng.uniform(min(tail, head) - 0.1 * span, max(tail, head) +
                     0.1 * span, 200000)).astype(dt)
    # add every edge and its neighbours
    ez = (-e if neg else e).astype(dt)
    z = np.concatenate([z, ez, np.nextafter(ez, dt(np.inf)),
                        np.nextafter(ez, dt(-np.inf))])
    want = np.floor((z.astype(np.float64) - tail) / width)
    u = -z if neg else z
    inside = (u >= e[0]) & (u < e[-1])
    got = np.searchsorted(e, u, side='right') - 1
    assert np.array_equal(inside, (want >= 0) & (want < S))
    assert np.array_equal(got[inside], want[inside].astype(np.int64))


def _fast_bin_f32(u, e):
    """The FP32 lookup's table-free path (Bins<float>::index_vec in
    csrc/phk_track.cuh), evaluated with the same float32 roundings:
    returns the index floor(u) and whether the path is taken."""
    f = np.float32
    S = len(e) - 1
    e0, eS = e[0], e[S]
    span = f(eS - e0)
    iw = f(f(S) / span) if span > 0 else f(0)
    m = f(f(2.0 ** -21) * f(f(f(abs(e0)) + f(abs(eS))) * iw + f(S) + f(2)))
    mg = m if m < f(0.25) else f(2)
    uu = (u.astype(np.float32) - e0).astype(np.float32) * iw
    fl = np.floor(uu)
    fr = uu - fl
    ok = (fr >= mg) & (fr <= f(1) - mg) & (fl >= 0) & (fl < S)
    return fl.astype(np.int64), ok, mg


@pytest.mark.parametrize('cuts,S', [((-0.69, 0.69), 500), ((-0.69, 0.69), 1000),
                                    ((-0.69, 0.69), 100), ((-0.31, 0.05), 7),
                                    ((0.2, -0.2), 13), ((-3e-3, 1e-2), 500),
                                    ((-1.1, 1.3), 1000), ((99.5, 100.5), 64),
                                    ((-1e-6, 1e-6), 1000), ((0.0, 2.0), 4096)])
def test_fp32_fast_bin_path_is_exact(cuts, S):
    """Wherever the table-free path is taken, floor(u) equals the
    reference's int(floor((z - tail) / width)) -- checked on random z, on
    every edge and its float neighbours, and on points a few ulps around
    every interior boundary, where the margin is what keeps it exact."""
    from pyheadtail_gb300 import _engine as E
    tail, head = cuts
    width = (head - tail) / float(S)
    e, neg = E.exact_edges(tail, width, S, 1)
    rng = np.random.RandomState(S + 7)
    span = abs(head - tail)
    z = rng.uniform(min(tail, head) - 0.1 * span, max(tail, head) + 0.1 * span,
                    400000).astype(np.float32)
    z = np.concatenate([z, rng.normal(0.5 * (tail + head), 0.2 * span,
                                      400000).astype(np.float32)])
    ez = (-e if neg else e).astype(np.float32)
    near = [ez]
    lo, hi = ez.copy(), ez.copy()
    for _ in range(8):
        lo = np.nextafter(lo, np.float32(-np.inf))
        hi = np.nextafter(hi, np.float32(np.inf))
        near += [lo, hi]
    z = np.concatenate([z] + near)
    want = np.floor((z.astype(np.float64) - tail) / width)
    u = -z if neg else z
    k, ok, mg = _fast_bin_f32(u, e)
    inside = (want >= 0) & (want < S)
    assert np.all(inside[ok])
    assert np.array_equal(k[ok], want[ok].astype(np.int64))
    if mg < 0.25 and span / S > 1e-5:
        # the fast path serves all but particles within mg of an edge
        assert ok[:800000].mean() > 1 - 4 * float(mg) - 0.25, ok.mean()


def _edges_uniform_f32(e, mg):
    """Bins<float>::edges_uniform: every edge within mg of its uniform
    position, in the device's float32 roundings."""
    f = np.float32
    S = len(e) - 1
    span = f(e[S] - e[0])
    iw = f(f(S) / span) if span > 0 else f(0)
    u = (e.astype(np.float32) - e[0]).astype(np.float32) * iw
    return bool(np.all(np.abs(u - np.arange(S + 1, dtype=np.float32)) < mg))


@pytest.mark.parametrize('cuts,S', [((-0.69, 0.69), 500), ((-0.69, 0.69), 1000),
                                    ((-0.31, 0.05), 7), ((0.2, -0.2), 13),
                                    ((-1.1, 1.3), 1000), ((99.5, 100.5), 64),
                                    ((0.0, 2.0), 4096)])
def test_fp32_fast_bin_vote(cuts, S):
    """Uniform-bin tables pass the kernels' uniformity vote (so the
    table-free lookup is used for them); the edge tables of uniform-charge
    slicing (order statistics of z) fail it and keep the exact search."""
    from pyheadtail_gb300 import _engine as E
    tail, head = cuts
    e, neg = E.exact_edges(tail, (head - tail) / float(S), S, 1)
    _, _, mg = _fast_bin_f32(e, e)
    if mg < 0.25:
        assert _edges_uniform_f32(e, mg)
    rng = np.random.RandomState(S)
    ce = np.sort(rng.normal(0, 0.23, S + 1)).astype(np.float32)
    _, _, cmg = _fast_bin_f32(ce, ce)
    assert cmg >= 0.25 or not _edges_uniform_f32(ce, cmg)


def test_fp32_fast_bin_path_random_slicers():
    """The table-free path's margin over 60 seeded random uniform slicers
    (cuts anywhere in [-5, 5], spans 1e-4 .. 10, 1 .. 4096 slices, either
    orientation): wherever it is taken, on every edge and 4 neighbours
    either side and on random z, it gives the reference's index."""
    from pyheadtail_gb300 import _engine as E
    rng = np.random.RandomState(2024)
    taken = 0
    for _ in range(60):
        S = int(rng.choice([1, 2, 7, 50, 100, 500, 1000, 4096]))
        span = 10.0 ** rng.uniform(-4, 1)
        tail = rng.uniform(-5, 5)
        head = tail + span * (1 if rng.rand() < 0.8 else -1)
        width = (head - tail) / float(S)
        e, neg = E.exact_edges(tail, width, S, 1)
        ez = (-e if neg else e).astype(np.float32)
        near = [ez]
        lo, hi = ez.copy(), ez.copy()
        for _ in range(4):
            lo = np.nextafter(lo, np.float32(-np.inf))
            hi = np.nextafter(hi, np.float32(np.inf))
            near += [lo, hi]
        z = np.concatenate(near + [rng.uniform(min(tail, head) - 0.1 * span,
                                               max(tail, head) + 0.1 * span,
                                               20000).astype(np.float32)])
        want = np.floor((z.astype(np.float64) - tail) / width)
        k, ok, mg = _fast_bin_f32(-z if neg else z, e)
        if mg < 0.25:
            assert _edges_uniform_f32(e, mg), (tail, head, S)
        assert np.array_equal(k[ok], want[ok].astype(np.int64)), (tail, head, S)
        taken += int(ok.sum())
    assert taken > 0


def test_header_constants_match_binding():
    """Every status, dtype and size constant of the header has the same
    value in the Python binding."""
    from pyheadtail_gb300 import _native as N
    src = open(HEADER).read()
    defs = dict(re.findall(r'#define\s+(PHK_\w+)\s+\(?(-?\d+)\)?', src))
    for name in ('PHK_F64', 'PHK_F32', 'PHK_DEV_TIMEOUT',
                 'PHK_DEV_TIMEOUT_UNDRAINED', 'PHK_DEV_BAD_TABLE',
                 'PHK_MAX_OPS', 'PHK_MAX_DETUNERS', 'PHK_MAX_POLY',
                 'PHK_MAX_KICKS', 'PHK_MAX_SLICES', 'PHK_X', 'PHK_DP'):
        assert int(defs[name]) == getattr(N, name), name
    # device status values are distinct
    st = [int(defs[k]) for k in ('PHK_DEV_TIMEOUT', 'PHK_DEV_TIMEOUT_UNDRAINED',
                                 'PHK_DEV_BAD_TABLE')]
    assert len(set(st)) == 3


def test_track_plan_validation(lib):
    """phk_set_track_plan rejects out-of-range plans on the host and
    accepts the tuner's candidates; phk_last_track_launch reports -1
    before any launch in a process that has launched nothing."""
    from pyheadtail_gb300 import _native as N
    from pyheadtail_gb300 import tuning
    L = N.load(build_if_missing=False)
    for bad in ((2, -1, -1), (-2, -1, -1), (0, 1, -1), (0, 5, -1),
                (1, -1, 15), (1, -1, 228)):
        assert L.phk_set_track_plan(*bad) == -4, bad
        assert 'phk_set_track_plan' in N.last_error()
    for cand in tuning.CANDIDATES + [tuning.DEFAULT_PLAN]:
        assert L.phk_set_track_plan(*cand) == 0, cand
    assert L.phk_set_track_plan(-1, -1, -1) == 0
    v, s, m = ctypes.c_int32(7), ctypes.c_int32(7), ctypes.c_int32(7)
    assert L.phk_last_track_launch(ctypes.byref(v), ctypes.byref(s),
                                   ctypes.byref(m)) == 0
    assert L.phk_last_track_launch(None, ctypes.byref(s),
                                   ctypes.byref(m)) == -1


def test_tuning_disabled_leaves_plan_untouched(tmp_path):
    """With tuning off the engine never sets a plan; the cache key names
    the pass configuration."""
    from pyheadtail_gb300 import tuning
    assert not tuning.enabled()
    tuning.enable(cache_path=str(tmp_path / 'p.json'))
    try:
        assert tuning.enabled()
        assert tuning._load() == {}
    finally:
        tuning.enable(on=False)
    assert not tuning.enabled()


def test_misaligned_tables_rejected_on_host(lib):
    """The kernels read slice edges, z and the moment quantities with loads
    of the coordinate type: a pointer that is not aligned to it is an
    argument error on the host (PHK_EALIGN), never a launch."""
    from pyheadtail_gb300 import _native as N
    L = N.load(build_if_missing=False)
    c = N.Coords()
    for i, f in enumerate(('x', 'xp', 'y', 'yp', 'z', 'dp')):
        setattr(c, f, 4096 * (i + 1))
    c.n, c.dtype = 100, N.PHK_F64
    prog = N.Program()
    sl = N.Slicer()
    sl.n_slices, sl.edges = 10, 65536 + 4          # 4-byte aligned only
    acc = N.Accum()
    acc.slicer = sl
    acc.partials, acc.grid, acc.partials_len = 131072, 1, 30
    assert L.phk_track(ctypes.byref(prog), ctypes.byref(c), None,
                       ctypes.byref(acc), None) == -3
    assert 'edges' in N.last_error()
    ks = N.KickSet()
    ks.slicer = sl
    ks.n_kicks, ks.target[0], ks.quad[0], ks.kick[0] = 1, N.COORD_INDEX['xp'], -1, 262144
    assert L.phk_track(ctypes.byref(prog), ctypes.byref(c), ctypes.byref(ks),
                       None, None) == -3
    assert L.phk_kick(ctypes.byref(c), ctypes.byref(ks), None) == -3
    # FP32 coordinates need only 4-byte alignment of the edges: the same
    # slicer passes the check and the call stops at a later argument error
    # (no sums array), still before any launch
    q = (ctypes.c_void_p * 1)(4096)
    assert L.phk_slice_moments(ctypes.byref(sl), 4096, 100, N.PHK_F32, q, 1,
                               0, None, None, 16384, None) == -1
    assert 'sums' in N.last_error()
    noalloc_sl = N.Slicer()
    noalloc_sl.n_slices, noalloc_sl.edges = 10, 65536 + 4
    assert L.phk_slice_noalloc(ctypes.byref(noalloc_sl), ctypes.byref(c),
                               8192, 16384, 32768, None) == -3
    # phk_slice_moments: edges, z and quantities
    sums, counts = 8192, 16384
    assert L.phk_slice_moments(ctypes.byref(sl), 4096, 100, N.PHK_F64, q, 1,
                               0, None, sums, counts, None) == -3
    sl.edges = 65536
    assert L.phk_slice_moments(ctypes.byref(sl), 4096 + 4, 100, N.PHK_F64, q,
                               1, 0, None, sums, counts, None) == -3
    q[0] = 4096 + 4
    assert L.phk_slice_moments(ctypes.byref(sl), 4096, 100, N.PHK_F64, q, 1,
                               0, None, sums, counts, None) == -3
    assert 'quantity' in N.last_error()


def test_misaligned_buffers_of_merges_and_wakes_rejected_on_host(lib):
    """Outputs and tables of the merges and wake convolutions: a pointer
    not aligned to its element type is PHK_EALIGN on the host.  Every call
    below fails validation, so none reaches a launch."""
    from pyheadtail_gb300 import _native as N
    L = N.load(build_if_missing=False)
    acc = N.Accum()
    acc.slicer.n_slices, acc.slicer.edges = 10, 65536
    acc.partials, acc.grid, acc.partials_len = 131072 + 4, 1, 30
    assert L.phk_slice_finalize(ctypes.byref(acc), 8192, 16384, 24576, None,
                                None) == -3
    assert 'partials' in N.last_error()
    acc.partials = 131072
    assert L.phk_slice_finalize(ctypes.byref(acc), 8192 + 2, 16384, 24576,
                                None, None) == -3
    assert 'counts' in N.last_error()
    assert L.phk_slice_finalize(ctypes.byref(acc), 8192, 16384 + 4, 24576,
                                None, None) == -3
    assert L.phk_slice_finalize(ctypes.byref(acc), 8192, 16384, 24576,
                                32768 + 4, None) == -3
    assert 'moments_slot' in N.last_error()
    assert L.phk_slice_merge(8192, 2, 10, 16384 + 2, 24576, 32768, None,
                             None) == -3
    assert L.phk_slice_merge(8192, 2, 10, 16384, 24576, 32768 + 4, None,
                             None) == -3
    assert L.phk_batch_finalize(ctypes.byref(acc), 2, 8192 + 2, 16384, 24576,
                                32768, None, 0, None) == -3
    assert 'bunch_columns' in N.last_error()

    ws = N.WakeSet()
    ws.n_slices, ws.ring_len, ws.head, ws.n_kicks = 10, 4, 0, 1
    ws.out_dtype = N.PHK_F64
    ws.moments = 8192 + 4
    ws.kick[0].table, ws.kick[0].out = 16384, 24576
    ws.kick[0].n_lags = 1
    assert L.phk_wake(ctypes.byref(ws), None) == -3
    assert 'moments' in N.last_error()
    ws.moments = 8192
    ws.kick[0].table = 16384 + 4
    assert L.phk_wake(ctypes.byref(ws), None) == -3
    ws.kick[0].table = 16384
    ws.kick[0].out = 24576 + 4          # FP64 output, 4-byte aligned
    assert L.phk_wake(ctypes.byref(ws), None) == -3
    assert 'output' in N.last_error()
    assert L.phk_wake_batch(8192 + 4, 2, 10, 1, None) == -3

    prog = N.Program()
    b = N.Batch()
    b.n_bunches, b.n_units, b.n_columns, b.grid, b.threads = 1, 1, 1, 1, 256
    b.units, b.cta_first, b.programs = 8192 + 4, 16384, 24576
    b.programs_host = ctypes.pointer(prog)
    c = N.Coords()
    for i, f in enumerate(('x', 'xp', 'y', 'yp', 'z', 'dp')):
        setattr(c, f, 65536 * (i + 1))
    c.n, c.dtype = 100, N.PHK_F32
    assert L.phk_track_batch(ctypes.byref(b), ctypes.byref(c), None, None,
                             None) == -3
    assert 'units' in N.last_error()


def test_misaligned_charge_slicer_tables_rejected_on_host(lib):
    """Uniform-charge order statistics: histogram, key and segment tables
    not aligned to their element type are PHK_EALIGN on the host (every
    call below fails validation before a launch)."""
    from pyheadtail_gb300 import _native as N
    L = N.load(build_if_missing=False)
    z = 4096
    assert L.phk_charge_hist(z, 100, N.PHK_F64, -0.5, 0.5, 16, 8192 + 2,
                             16384, None) == -3
    assert L.phk_charge_hist(z, 100, N.PHK_F64, -0.5, 0.5, 16, 8192,
                             16384 + 4, None) == -3
    assert L.phk_charge_gather(z, 100, N.PHK_F64, -0.5, 0.5, 16, 8192,
                               16384 + 4, 24576, 32768, 40960, 49152,
                               None) == -3
    assert 'seg_off' in N.last_error()
    assert L.phk_charge_gather(z, 100, N.PHK_F64, -0.5, 0.5, 16, 8192,
                               16384, 24576, 32768, 40960 + 4, 49152,
                               None) == -3
    assert 'keys' in N.last_error()
    assert L.phk_charge_select(8192 + 4, 16384, 24576, 32768, 40960, 3,
                               49152, 57344, None) == -3
    assert L.phk_charge_select(8192, 16384, 24576, 32768, 40960, 3,
                               49152 + 4, 57344, None) == -3
    assert "out" in N.last_error()


def test_misaligned_status_word_rejected_on_host(lib):
    """The optional device status word of a program is updated with 32-bit
    atomics: a pointer not aligned to 4 bytes is PHK_EALIGN on the host."""
    from pyheadtail_gb300 import _native as N
    L = N.load(build_if_missing=False)
    prog = N.Program()
    prog.status = 8192 + 2
    c = N.Coords()
    for i, f in enumerate(('x', 'xp', 'y', 'yp', 'z', 'dp')):
        setattr(c, f, 4096 * (i + 1))
    c.n, c.dtype = 100, N.PHK_F64
    assert L.phk_track(ctypes.byref(prog), ctypes.byref(c), None, None,
                       None) == -3
    assert 'status' in N.last_error()
    w = N.WakeTC()
    w.n_slices, w.n_groups, w.n_kicks = 10, 1, 1
    w.group_lags[0] = 2
    w.status = 8192 + 2
    a_el, p_el = ctypes.c_int64(), ctypes.c_int64()
    assert L.phk_wake_tc_plan(ctypes.byref(w), ctypes.byref(a_el),
                              ctypes.byref(p_el)) == -3
