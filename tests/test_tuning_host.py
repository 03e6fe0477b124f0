"""Host logic of the single-bunch autotuner (no GPU): which timed plans
compete, what the cache holds, and when the default plan is used.

The native calls, CUDA events and device queries are replaced by fakes:
a fake launch reports the plan it "ran" through phk_last_track_launch the
way the library does when a plan's shared memory does not fit (another
kernel variant, or fewer ring stages)."""
import json
import types

import pytest
import torch

from pyheadtail_gb300 import _native as N
from pyheadtail_gb300 import tuning


class _Fake(object):
    """phk_set_track_plan / phk_track / phk_last_track_launch stand-ins and a
    device clock that each launch advances by the asked plan's time."""

    def __init__(self, times, launched):
        self.times = times          # asked plan -> ms per launch
        self.launched = launched    # asked plan -> (variant, stages) run
        self.plan = tuning.DEFAULT_PLAN
        self.clock = 0.0
        self.tracks = 0
        self.plans_set = []
        self.x_ptrs = set()

    def call(self, name, *args):
        if name == 'phk_set_track_plan':
            self.plan = tuple(args)
            self.plans_set.append(self.plan)
        elif name == 'phk_track':
            self.tracks += 1
            self.x_ptrs.add(args[1]._obj.x)
            self.clock += self.times.get(self.plan, 1.0)
        elif name == 'phk_last_track_launch':
            v, s = self.launched.get(self.plan, self.plan[:2])
            args[0]._obj.value = v
            args[1]._obj.value = s
            args[2]._obj.value = 1024 * max(self.plan[2], 0)
        else:
            raise AssertionError('unexpected native call ' + name)
        return 0

    def event(self, enable_timing=False):
        fake = self

        class Ev(object):
            def record(self):
                self.t = fake.clock

            def elapsed_time(self, other):
                return other.t - self.t
        return Ev()


def _engine(n=4096):
    c = {k: torch.zeros(n, dtype=torch.float32)
         for k in ('x', 'xp', 'y', 'yp', 'z', 'dp')}
    beam = types.SimpleNamespace(_c=c, _device=0, macroparticlenumber=n)
    return types.SimpleNamespace(beam=beam)


def _ops():
    return [types.SimpleNamespace(kind=1, flags=0, detuners=[]),
            types.SimpleNamespace(kind=3, flags=2, detuners=[1, 2])]


@pytest.fixture
def fake(monkeypatch, tmp_path):
    times = {c: 1.0 for c in tuning.CANDIDATES}
    times[(0, 3, 72)] = 0.5                 # the fastest plan that fits
    times[(1, 2, 56)] = 0.1                 # faster, but fell back to variant 0
    times[(0, 4, 56)] = 0.2                 # faster, but ran with two stages
    launched = {(1, 2, 56): (0, 2), (0, 4, 56): (0, 2)}
    f = _Fake(times, launched)
    monkeypatch.setattr(tuning.N, 'call', f.call)
    monkeypatch.setattr(tuning.torch.cuda, 'Event', f.event)
    monkeypatch.setattr(tuning.torch.cuda, 'synchronize', lambda: None)
    monkeypatch.setattr(tuning.torch.cuda, 'is_current_stream_capturing',
                        lambda: False)
    monkeypatch.setattr(tuning.torch.cuda, 'get_device_name',
                        lambda d=None: 'FAKE GB300')
    monkeypatch.setattr(tuning, '_state', {'enabled': False,
                                           'cache_path': None, 'cache': None,
                                           'tuned': {}})
    f.cache_path = str(tmp_path / 'plans.json')
    return f


def _plan(engine):
    return tuning.plan_for(engine, N.Program(), N.Coords(), None, None,
                           _ops(), None, None, None)


def test_disabled_gives_default_and_launches_nothing(fake):
    assert _plan(_engine()) == tuning.DEFAULT_PLAN
    assert fake.tracks == 0


def test_only_plans_that_launched_as_asked_compete(fake):
    tuning.enable(cache_path=fake.cache_path)
    eng = _engine()
    assert _plan(eng) == (0, 3, 72)
    # every candidate timed (one untimed + three timed launches each),
    # the plan reset to the default afterwards
    assert fake.tracks == 4 * len(tuning.CANDIDATES)
    assert fake.plans_set[-1] == tuning.DEFAULT_PLAN
    with open(fake.cache_path) as f:
        cache = json.load(f)
    (key, entry), = cache.items()
    assert entry['plan'] == [0, 3, 72]
    assert entry['ms'] == pytest.approx(0.5)
    assert '1,2,56' not in entry['candidates']
    assert '0,4,56' not in entry['candidates']
    assert len(entry['candidates']) == len(tuning.CANDIDATES) - 2
    assert 'FAKE GB300' in key and '4096' in key
    # the launches ran on scratch copies, never on the beam's arrays
    assert len(fake.x_ptrs) == 1
    assert eng.beam._c['x'].data_ptr() not in fake.x_ptrs


def test_winner_is_reused_in_process_and_from_the_cache_file(fake):
    tuning.enable(cache_path=fake.cache_path)
    _plan(_engine())
    n = fake.tracks
    assert _plan(_engine()) == (0, 3, 72)
    assert fake.tracks == n                 # in-process table
    tuning.enable(cache_path=fake.cache_path)   # a new process, same file
    tuning._state['tuned'].clear()
    assert _plan(_engine()) == (0, 3, 72)
    assert fake.tracks == n                 # read back, not re-timed
    assert tuning.timings()[next(iter(tuning.timings()))]['plan'] == [0, 3, 72]


def test_other_configurations_are_tuned_separately(fake):
    tuning.enable(cache_path=fake.cache_path)
    _plan(_engine(4096))
    n = fake.tracks
    _plan(_engine(8192))
    assert fake.tracks == 2 * n
    assert len(tuning.timings()) == 2


def test_capture_in_progress_uses_the_default_untimed(fake, monkeypatch):
    tuning.enable(cache_path=fake.cache_path)
    monkeypatch.setattr(tuning.torch.cuda, 'is_current_stream_capturing',
                        lambda: True)
    assert _plan(_engine()) == tuning.DEFAULT_PLAN
    assert fake.tracks == 0


def test_unreadable_cache_file_is_retuned(fake):
    with open(fake.cache_path, 'w') as f:
        f.write('{not json')
    tuning.enable(cache_path=fake.cache_path)
    assert _plan(_engine()) == (0, 3, 72)
    with open(fake.cache_path) as f:
        assert json.load(f)                 # rewritten whole


def test_launch_report_reads_variant_and_stages(fake):
    fake.plan = (1, 3, 72)
    assert tuning._last_launch() == (1, 3)
