"""TransverseDamper's per-plane entry points on the host (no GPU):
track_horizontal / track_vertical / track_all (transverse_damper.py:68-88)
enqueue exactly the statistics pass and DAMPER op that a damper of only
those planes enqueues from track (the form the GPU tests check against the
oracle), and a plane without a damping rate raises TypeError."""
import numpy as np
import pytest

torch = pytest.importorskip('torch')

from pyheadtail_gb300.feedback.transverse_damper import TransverseDamper  # noqa: E402
from pyheadtail_gb300.general.printers import SilentPrinter  # noqa: E402


class _Engine(object):
    def __init__(self):
        self.ops = []

    def enqueue(self, op):
        self.ops.append(op)


class _Beam(object):
    """What the damper touches: the device, launch_stats, the engine."""

    def __init__(self):
        self._device = torch.device('cpu')
        self._engine = _Engine()
        self.stats = []

    def launch_stats(self, rec, order=1, mask=0, means=None):
        self.stats.append((order, mask))


def _trace(damper, method):
    b = _Beam()
    for _ in range(2):
        getattr(damper, method)(b)
    ops = [(op.kind, op.flags, sorted(op.p.items()),
            sorted((k, float(v)) for k, v in op.pf.items()))
           for op in b._engine.ops]
    return ops, b.stats


def _damper(rx, ry, **kw):
    return TransverseDamper(rx, ry, printer=SilentPrinter(), **kw)


@pytest.mark.parametrize('kw', [{}, dict(phase=30, local_beta_function=50.)])
def test_per_plane_entry_points_match_single_plane_dampers(kw):
    both = _damper(40, 60, **kw)
    assert _trace(both, 'track_horizontal') == _trace(_damper(40, 0, **kw),
                                                      'track')
    assert _trace(both, 'track_vertical') == _trace(_damper(0, 60, **kw),
                                                    'track')
    assert _trace(both, 'track_all') == _trace(both, 'track')
    ops, stats = _trace(both, 'track_all')
    assert len(ops) == 2 and len(stats) == 2


def test_unset_plane_raises():
    with pytest.raises(TypeError):
        _damper(0, 60).track_horizontal(_Beam())
    with pytest.raises(TypeError):
        _damper(40, 0).track_all(_Beam())
    b = _Beam()
    _damper(0, 0).track(b)
    assert not b._engine.ops and not b.stats
