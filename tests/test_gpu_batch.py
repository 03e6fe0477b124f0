"""Batched form on the GPU: many bunches of uneven sizes, each with its own
chromaticity and intensity, tracked by one persistent launch per turn.

* against the oracle, bunch by bunch (the oracle is bit-identical to the
  reference on the golden fixtures): slice counts bit-exact, coordinates
  and slice centroids within 1e-12 of their RMS;
* against the single-bunch GPU path in both precisions;
* CUDA-graph replay against eager turns (bit-identical);
* a multi-turn wake (ring of 4 stored turns);
* the autotuner, and the device-side check of the unit table.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip('torch')

COORDS = ('x', 'xp', 'y', 'yp', 'z', 'dp')
SIZES = [1, 3, 1001, 4099, 20000, 65543]


def rms_err(got, ref):
    got = np.asarray(got, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    if ref.size == 0:
        return 0.
    scale = np.sqrt(np.mean(ref**2)) or 1.
    return float(np.max(np.abs(got - ref)) / scale)


def _specs(sizes, n_turns, rw_turns=0, seed=40):
    import cases as C
    rng = np.random.default_rng(seed)
    specs = []
    for b, n in enumerate(sizes):
        q = float(rng.uniform(-5, 15))
        intensity = float(rng.uniform(5e10, 2e11))
        sources = [C.resonator()]
        if rw_turns:
            sources.append(C.resistive_wall(n_turns_wake=rw_turns))
        specs.append(dict(
            beam=C.beam_params(n, seed + b, intensity=intensity),
            n_turns=n_turns,
            elements=[C.smooth_transverse(chroma=[q, q]), C.rf(),
                      C.wake(C.slicer(50), *sources)]))
    return specs


def _coords(spec):
    from oracle import cases as OC
    return OC.make_beam(spec['beam']).coords()


def _batched(specs, coords, precision='fp64', **kw):
    import gpu_cases as G
    from pyheadtail_gb300.batch import BatchedTurn, BunchBatch
    beams, maps = [], []
    for spec, c in zip(specs, coords):
        beam = G.make_beam(spec['beam'], c, precision=precision)
        beams.append(beam)
        maps.append([el for _, el in G.make_elements(spec, beam)])
    batch = BunchBatch(beams)
    return beams, BatchedTurn(batch, maps, **kw)


@pytest.fixture(scope='module')
def lib():
    from pyheadtail_gb300 import _native as N
    return N.load()


def test_batch_matches_oracle_bunch_by_bunch(lib):
    from oracle import cases as OC
    T = 6
    specs = _specs(SIZES, T)
    coords = [_coords(s) for s in specs]
    beams, turn = _batched(specs, coords,
                           config={'threads': 256, 'unit_tiles': 2,
                                   'ctas_per_sm': 2})
    turn.track(T)
    torch.cuda.synchronize()
    assert turn.read_status() == 0
    j = 2                                # the wake is element 2 of each map
    for b, spec in enumerate(specs):
        ob = OC.make_beam(spec['beam'])
        ref = OC.run(spec, ob, n_turns=T, record_turns=(T - 1,))
        got = beams[b].coords_numpy()
        for k in COORDS:
            assert rms_err(got[k], ref['t%d_%s' % (T - 1, k)]) <= 1e-12, \
                (b, k)
        p = 't%d_e%d_' % (T - 1, j)
        np.testing.assert_array_equal(turn.counts[b].cpu().numpy(),
                                      ref[p + 'counts'])
        assert rms_err(turn.mean_x[b].cpu().numpy(), ref[p + 'mean_x']) \
            <= 1e-12
        assert rms_err(turn.mean_y[b].cpu().numpy(), ref[p + 'mean_y']) \
            <= 1e-12


def test_batch_large_bunches_match_oracle(lib):
    """Bunches at the top of the batched workload's size range (1e6
    macroparticles, as the largest of its log-uniform draw in [1e4, 1e6])
    beside mid-size and ragged ones, each with its own Q' and intensity:
    the oracle bunch by bunch after 6 turns, counts exact, coordinates and
    slice means within 1e-12."""
    from oracle import cases as OC
    T = 6
    specs = _specs([1000000, 370001, 12345], T, seed=90)
    coords = [_coords(s) for s in specs]
    beams, turn = _batched(specs, coords)
    turn.track(T)
    torch.cuda.synchronize()
    assert turn.read_status() == 0
    p = 't%d_e2_' % (T - 1)
    for b, spec in enumerate(specs):
        ref = OC.run(spec, OC.make_beam(spec['beam']), n_turns=T,
                     record_turns=(T - 1,))
        got = beams[b].coords_numpy()
        for k in COORDS:
            assert rms_err(got[k], ref['t%d_%s' % (T - 1, k)]) <= 1e-12, \
                (b, k)
        np.testing.assert_array_equal(turn.counts[b].cpu().numpy(),
                                      ref[p + 'counts'])
        assert rms_err(turn.mean_x[b].cpu().numpy(), ref[p + 'mean_x']) \
            <= 1e-12
        assert rms_err(turn.mean_y[b].cpu().numpy(), ref[p + 'mean_y']) \
            <= 1e-12


@pytest.mark.parametrize('precision,tol', [('fp64', 1e-12), ('fp32', 1e-5)])
def test_batch_matches_single_bunch_path(lib, precision, tol):
    import gpu_cases as G
    T = 8
    specs = _specs(SIZES, T, seed=60)
    coords = [_coords(s) for s in specs]
    beams, turn = _batched(specs, coords, precision=precision)
    turn.track(T)
    for b, (spec, c) in enumerate(zip(specs, coords)):
        single = G.make_beam(spec['beam'], c, precision=precision)
        els = [el for _, el in G.make_elements(spec, single)]
        for _ in range(T):
            for el in els:
                el.track(single)
        want = single.coords_numpy()
        got = beams[b].coords_numpy()
        for k in COORDS:
            assert rms_err(got[k], want[k]) <= tol, (precision, b, k)
        ss = els[-1].slice_set_deque[0]
        np.testing.assert_array_equal(
            turn.counts[b].cpu().numpy(),
            ss.n_macroparticles_per_slice.cpu().numpy())


def test_graph_replay_equals_eager_turns(lib):
    T = 7
    specs = _specs([5, 777, 30001], T, seed=80)
    coords = [_coords(s) for s in specs]
    cfg = {'threads': 128, 'unit_tiles': 4, 'ctas_per_sm': 1}
    beams_e, eager = _batched(specs, coords, config=cfg, warmup_turns=10**9)
    eager.track(T)
    beams_g, graph = _batched(specs, coords, config=cfg, warmup_turns=2)
    graph.track(T)
    assert graph._graph is not None and eager._graph is None
    for be, bg in zip(beams_e, beams_g):
        ce, cg = be.coords_numpy(), bg.coords_numpy()
        for k in COORDS:
            np.testing.assert_array_equal(ce[k], cg[k])


def test_multiturn_wake_ring(lib):
    import gpu_cases as G
    T = 9
    specs = _specs([2000, 513, 12345], T, rw_turns=4, seed=90)
    coords = [_coords(s) for s in specs]
    beams, turn = _batched(specs, coords, warmup_turns=3)
    turn.track(T)
    assert turn.R == 4 and turn._graph is not None
    for b, (spec, c) in enumerate(zip(specs, coords)):
        single = G.make_beam(spec['beam'], c)
        els = [el for _, el in G.make_elements(spec, single)]
        for _ in range(T):
            for el in els:
                el.track(single)
        want, got = single.coords_numpy(), beams[b].coords_numpy()
        for k in COORDS:
            assert rms_err(got[k], want[k]) <= 1e-12, (b, k)


def test_autotune_picks_and_caches_a_shape(lib):
    import os
    from pyheadtail_gb300 import batch as B
    specs = _specs([50000, 20000, 7], 1, seed=100)
    coords = [_coords(s) for s in specs]
    path = os.path.join(os.path.dirname(B.default_cache_path()),
                        'test_autotune.json')
    try:
        beams, turn = _batched(specs, coords, autotune=True,
                               cache_path=path, precision='fp32')
        assert turn.config['threads'] in B.THREADS
        assert len(B.load_cache(path)) == 1
        before = [b.coords_numpy()['x'].copy() for b in beams]
        turn.track(2)                  # tuning ran on a scratch copy
        assert any(not np.array_equal(b.coords_numpy()['x'], x0)
                   for b, x0 in zip(beams, before) if len(x0) > 1)
    finally:
        if os.path.exists(path):
            os.remove(path)


def test_unit_table_checked_on_device(lib):
    """A unit past the end of the coordinates is skipped by the kernel,
    which reports PHK_DEV_BAD_TABLE instead of touching memory."""
    import ctypes
    from pyheadtail_gb300 import _native as N
    from pyheadtail_gb300 import batch as B
    specs = _specs([64, 64], 1, seed=110)
    coords = [_coords(s) for s in specs]
    beams, turn = _batched(specs, coords,
                           config={'threads': 256, 'unit_tiles': 2,
                                   'ctas_per_sm': 1})
    p = turn._p
    plan = dict(p['plan'])
    units = plan['units'].copy()
    units[-1, 1] = turn.batch.total + 4096            # beyond the arrays
    plan['units'] = units
    p = dict(p, units=B.unit_table(plan, turn.batch.device))
    before = {k: v.clone() for k, v in turn.batch.storage.items()}
    b = turn._batch_struct(p)
    N.call('phk_track_batch', ctypes.byref(b),
           ctypes.byref(turn.batch.coords_struct()), None, None, None)
    torch.cuda.synchronize()
    assert turn.read_status() == N.PHK_DEV_BAD_TABLE
    last = int(plan['units'][-1, 0])
    for k in COORDS:    # the skipped unit's particles are untouched
        assert torch.equal(before[k][last:], turn.batch.storage[k][last:])
