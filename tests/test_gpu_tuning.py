"""Autotuner of the FP32 single-bunch pass (pyheadtail_gb300.tuning).

On the large single bunch's physics (Q' = 2, amplitude detuning, RF, 1000
slices, resonator + 50-turn resistive wall), reduced to 2e6
macroparticles: the first turn times the candidate plans and caches the
winner; later turns, and a fresh process state reading the cache file,
launch exactly the cached plan (checked with phk_last_track_launch); a
plan written into the cache by hand is honoured; tuned turns give the
same coordinates, bit for bit, as turns with the default plan."""
import ctypes
import json

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip('torch')

N_MP = 2 * 10**6


def _spec():
    import cases as C
    return dict(beam=C.beam_params(N_MP, 5), n_turns=3, elements=[
        C.smooth_transverse(chroma=[2., 2.],
                            amplitude=[1e-11, 1e-11, -5e-12]),
        C.rf(), C.wake(C.slicer(1000), C.resonator(),
                       C.resistive_wall(n_turns_wake=50))])


def _last_launch():
    from pyheadtail_gb300 import _native as N
    v, s, m = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
    N.call('phk_last_track_launch', ctypes.byref(v), ctypes.byref(s),
           ctypes.byref(m))
    return v.value, s.value, m.value


def _turns(spec, coords, n_turns, after_each=None):
    import gpu_cases as G
    beam = G.make_beam(spec['beam'], coords, precision='fp32')
    els = [el for _, el in G.make_elements(spec, beam)]
    for t in range(n_turns):
        for el in els:
            el.track(beam)
        if after_each is not None:
            after_each(t)
    beam.mean_x()                       # runs any pending pass
    return {k: getattr(beam, k).cpu().numpy().copy()
            for k in ('x', 'xp', 'y', 'yp', 'z', 'dp')}


@pytest.fixture
def fresh_tuning(tmp_path):
    from pyheadtail_gb300 import _native as N
    from pyheadtail_gb300 import tuning
    path = str(tmp_path / 'plans.json')
    tuning._state['tuned'] = {}
    tuning.enable(cache_path=path)
    yield tuning, path
    tuning.enable(on=False)
    tuning._state['tuned'] = {}
    N.call('phk_set_track_plan', -1, -1, -1)


def _fused_entry(cache):
    """The cache entry of the fused turn pass (the one with pending kicks
    and an accumulation)."""
    keys = [k for k in cache if not k.split('|')[4] == 'none'
            and not k.split('|')[5] == 'none']
    assert len(keys) == 1, list(cache)
    return keys[0]


def test_pick_cached_and_honoured(fresh_tuning):
    from oracle import cases as OC
    from pyheadtail_gb300 import _native as N
    tuning, path = fresh_tuning
    spec = _spec()
    coords = OC.make_beam(spec['beam']).coords()

    launches = []
    tuned = _turns(spec, coords, 4,
                   after_each=lambda t: launches.append(_last_launch()))
    with open(path) as f:
        cache = json.load(f)
    key = _fused_entry(cache)
    plan = tuple(cache[key]['plan'])
    assert plan in tuning.CANDIDATES
    assert cache[key]['ms'] > 0
    # the last launch of each turn is the fused pass of the wake element
    # (from the second turn on: with the pending kicks of the previous one)
    want_variant = 1 if plan[0] == 1 else 0
    for v, s, m in launches[1:]:
        assert v == want_variant
        if plan[1] >= 0 and want_variant == 1:
            assert s == plan[1]
        if plan[2] > 0:
            assert 0 < m <= plan[2] * 1024
    # no second timing: the candidates ran once for each pass configuration
    n_entries = len(cache)
    _turns(spec, coords, 2)
    with open(path) as f:
        assert len(json.load(f)) == n_entries

    # a fresh process state reads the cache; a hand-written pick of the
    # streaming kernel with two stages (68 KB at 1000 + 1000 slices) is
    # honoured
    cache[key]['plan'] = [1, 2, 72]
    with open(path, 'w') as f:
        json.dump(cache, f)
    tuning._state['tuned'] = {}
    tuning.enable(cache_path=path)
    launches2 = []
    forced = _turns(spec, coords, 4,
                    after_each=lambda t: launches2.append(_last_launch()))
    for v, s, m in launches2[1:]:
        assert (v, s) == (1, 2) and 0 < m <= 72 * 1024
    # and the tile-shared kernel without a TMA ring
    cache[key]['plan'] = [0, 0, 72]
    with open(path, 'w') as f:
        json.dump(cache, f)
    tuning._state['tuned'] = {}
    tuning.enable(cache_path=path)
    launches3 = []
    tile = _turns(spec, coords, 4,
                  after_each=lambda t: launches3.append(_last_launch()))
    for v, s, m in launches3[1:]:
        assert (v, s) == (0, 0) and 0 < m <= 72 * 1024

    # every plan gives the same coordinates as the default
    tuning.enable(on=False)
    N.call('phk_set_track_plan', -1, -1, -1)
    default = _turns(spec, coords, 4)
    for k in default:
        for other in (tuned, forced, tile):
            assert np.array_equal(other[k].view(np.uint32),
                                  default[k].view(np.uint32)), k
