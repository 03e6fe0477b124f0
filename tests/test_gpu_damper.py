"""TransverseDamper on the GPU.

The plain FP64 form replays the reference's own fixtures (damper_*.npz) in
test_gpu_parity.py.  Here:
* the FP32 form with a damper after a wake stays within the precision
  form's bars of the FP64 oracle;
* a turn with a damper is captured into a CUDA graph (the damper's
  statistics pass and the op that reads its device means) and replays to
  the same coordinates, bit for bit, as the eager turns.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip('torch')

COORDS = ('x', 'xp', 'y', 'yp', 'z', 'dp')


@pytest.fixture(scope='module')
def lib():
    from pyheadtail_gb300 import _native
    return _native.load()


def test_fp32_damper_against_oracle(lib):
    import cases as C
    import gpu_cases as G
    from oracle import cases as OC
    spec = dict(C.CASES['damper_resistive'])
    spec['beam'] = C.beam_params(20000, 26)
    ob = OC.make_beam(spec['beam'])
    coords = ob.coords()
    T = 30
    ref = OC.run(spec, ob, n_turns=T, record_turns=(T - 1,))
    beam = G.make_beam(spec['beam'], coords, precision='fp32')
    rec = G.run(spec, beam, n_turns=T, record_turns=(T - 1,))
    errs = []
    for k in COORDS:
        g = np.asarray(rec['t%d_%s' % (T - 1, k)], np.float64)
        r = ref['t%d_%s' % (T - 1, k)]
        errs.append(np.abs(g - r) / np.sqrt(np.mean(r**2)))
    errs = np.concatenate(errs)
    rms, mx = float(np.sqrt(np.mean(errs**2))), float(errs.max())
    print('FP32 damper after %d turns: coords rms %.3g max %.3g' % (T, rms, mx))
    assert rms <= 1e-4 and mx <= 3e-2


class _Count(object):
    """Counts the turns of a one-turn map (host side only)."""

    def __init__(self):
        self.n = 0

    def track(self, beam):
        self.n += 1


def test_damper_turn_graph_replay(lib):
    import cases as C
    import gpu_cases as G
    from oracle import cases as OC
    from pyheadtail_gb300.turngraph import TurnGraph
    spec = dict(C.CASES['damper_resistive'])
    spec['beam'] = C.beam_params(50000, 26)
    coords = OC.make_beam(spec['beam']).coords()
    eager = G.make_beam(spec['beam'], coords)
    els = [el for _, el in G.make_elements(spec, eager)]
    graphed = G.make_beam(spec['beam'], coords)
    count = _Count()
    gels = [el for _, el in G.make_elements(spec, graphed)] + [count]
    tg = TurnGraph(gels, graphed, warmup_turns=3).capture()
    # the capture itself ran turns_per_graph turns of host code
    warm = count.n - tg.turns_per_graph
    assert warm >= 3
    for _ in range(warm):
        for el in els:
            el.track(eager)
    tg.replay(3)
    for _ in range(3 * tg.turns_per_graph):
        for el in els:
            el.track(eager)
    torch.cuda.synchronize()
    for k in COORDS:
        assert torch.equal(getattr(eager, k), getattr(graphed, k)), k


def test_streamed_turns_match_eager(lib):
    """turngraph.StreamedTurns (copy of one bunch overlapped with the turn
    of the previous one, two beams in turn) gives, for every pushed bunch,
    the centroid an eager loop gives after loading the same coordinates and
    tracking one turn (zero intensity: no wake kick carries over)."""
    import cases as C
    import gpu_cases as G
    from oracle import cases as OC
    from pyheadtail_gb300.turngraph import StreamedTurns
    spec = dict(C.CASES['c1_full'])
    spec['beam'] = C.beam_params(20000, 0, intensity=0.)
    bunches = []
    for seed in range(5):
        c = OC.make_beam(C.beam_params(20000, 100 + seed)).coords()
        bunches.append({k: torch.from_numpy(v).pin_memory()
                        for k, v in c.items()})

    def make(k):
        b = G.make_beam(spec['beam'], OC.make_beam(spec['beam']).coords())
        return b, [el for _, el in G.make_elements(spec, b)]
    st = StreamedTurns(make, n_slots=2)
    got = []
    for h in bunches:
        r = st.push(h)
        if r is not None:
            got.append(r)
    got += st.drain()
    want = []
    for h in bunches:
        b = G.make_beam(spec['beam'], {k: v.numpy() for k, v in h.items()})
        for _, el in G.make_elements(spec, b):
            el.track(b)
        want.append((b.mean_x(), b.mean_y()))
    assert len(got) == len(want)
    for g, w in zip(got, want):
        assert abs(g[0] - w[0]) <= 1e-12 * 1e-3 and \
            abs(g[1] - w[1]) <= 1e-12 * 1e-3, (g, w)
