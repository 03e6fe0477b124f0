"""Autotuner of the FP32 single-bunch pass (phk_track with float
coordinates): kernel variant, TMA ring stages and shared-memory budget.

No counterpart in the reference (its elements run NumPy loops).  With
tuning enabled, the first eager pass of each configuration -- device,
number of particles, element-program shape, slicings, pending kicks --
times every candidate launch plan on scratch copies of the coordinates
(the same program, kick tables and slicings; the beam is not touched),
keeps the fastest and stores it in a JSON cache; every later pass of that
configuration sets the plan (phk_set_track_plan) before its launch, so a
turn captured as a CUDA graph records it.  All plans give identical
results; only the time differs.

    from pyheadtail_gb300 import tuning
    tuning.enable()            # or tuning.enable(cache_path=...)
"""
import ctypes
import json
import os

import numpy as np
import torch

from . import _native as N

DEFAULT_PLAN = (-1, -1, -1)

# (variant, stages, shared-memory KB): the tile-shared kernel (0) with the
# TMA ring of 0 / 2 / 3 / 4 stages at four, three or two CTAs per SM, and
# the streaming kernel (1) with 2-4 stages per warp
CANDIDATES = ([(0, s, kb) for s in (0, 2, 3, 4) for kb in (56, 72, 108)] +
              [(1, s, kb) for s in (2, 3, 4) for kb in (56, 72, 108)])

_state = {'enabled': False, 'cache_path': None, 'cache': None,
          'tuned': {}}


def default_cache_path():
    return os.path.join(os.path.expanduser('~'), '.cache', 'pyheadtail_gb300',
                        'track_plans.json')


def enable(cache_path=None, on=True):
    """Turn tuning on (or off) for the process."""
    _state['enabled'] = bool(on)
    _state['cache_path'] = cache_path or default_cache_path()
    _state['cache'] = None


def enabled():
    return _state['enabled']


def _load():
    if _state['cache'] is None:
        p = _state['cache_path']
        try:
            with open(p) as f:
                _state['cache'] = json.load(f)
        except (OSError, ValueError):
            _state['cache'] = {}
    return _state['cache']


def _store():
    p = _state['cache_path']
    try:
        os.makedirs(os.path.dirname(p), exist_ok=True)
        tmp = p + '.tmp'
        with open(tmp, 'w') as f:
            json.dump(_state['cache'], f, indent=1, sort_keys=True)
        os.replace(tmp, p)
    except OSError:
        pass


def config_key(beam, ops, kick, acc):
    """The configuration a plan is tuned for."""
    dev = torch.cuda.get_device_name(beam._device)
    shape = ','.join('%d:%d' % (o.kind, o.flags) for o in ops)
    dets = ','.join('%d' % len(o.detuners) for o in ops)
    pk = ('none' if kick is None else '%d:%d' % (
        kick.dslicer.n_slices, len(kick.kicks)))
    ac = 'none' if acc is None else '%d' % acc.dslicer.n_slices
    return '|'.join([dev, str(beam.macroparticlenumber), shape, dets, pk, ac])


def plan_for(engine, prog, coords, ks, ac, ops, kick, acc, stream):
    """The plan to launch this pass with: the cached winner, after timing
    the candidates once if tuning is on; the default otherwise."""
    if not _state['enabled']:
        return DEFAULT_PLAN
    key = config_key(engine.beam, ops, kick, acc)
    plan = _state['tuned'].get(key)
    if plan is not None:
        return plan
    cache = _load()
    if key in cache:
        plan = tuple(cache[key]['plan'])
        _state['tuned'][key] = plan
        return plan
    if torch.cuda.is_current_stream_capturing():
        return DEFAULT_PLAN
    plan, ms, every = _time_candidates(engine, prog, coords, ks, ac, stream)
    cache[key] = {'plan': list(plan), 'ms': ms,
                  'candidates': {'%d,%d,%d' % c: t for c, t in every.items()}}
    _state['tuned'][key] = plan
    _store()
    return plan


def _last_launch():
    v, s, m = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
    N.call('phk_last_track_launch', ctypes.byref(v), ctypes.byref(s),
           ctypes.byref(m))
    return v.value, s.value


def _time_candidates(engine, prog, coords, ks, ac, stream, reps=3):
    beam = engine.beam
    scratch = {k: t.clone() for k, t in beam._c.items()}
    c = N.Coords()
    ctypes.memmove(ctypes.byref(c), ctypes.byref(coords), ctypes.sizeof(N.Coords))
    c.x, c.xp, c.y = (scratch['x'].data_ptr(), scratch['xp'].data_ptr(),
                      scratch['y'].data_ptr())
    c.yp, c.z, c.dp = (scratch['yp'].data_ptr(), scratch['z'].data_ptr(),
                       scratch['dp'].data_ptr())
    results = {}
    try:
        for cand in CANDIDATES:
            N.call('phk_set_track_plan', *cand)
            times = []
            for it in range(reps + 1):
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record()
                N.call('phk_track', ctypes.byref(prog), ctypes.byref(c),
                       ctypes.byref(ks) if ks is not None else None,
                       ctypes.byref(ac) if ac is not None else None, stream)
                e1.record()
                torch.cuda.synchronize()
                if it:
                    times.append(e0.elapsed_time(e1))
            # a plan whose shared memory does not fit runs the other kernel
            # or fewer ring stages: only plans that launched as asked compete
            v, s = _last_launch()
            if v == cand[0] and (cand[1] < 0 or s == cand[1]):
                results[cand] = float(np.median(times))
    finally:
        N.call('phk_set_track_plan', *DEFAULT_PLAN)
    del scratch
    best = min(results, key=results.get)
    return best, results[best], results


def timings():
    """Every tuned configuration of the cache: {key: {'plan', 'ms',
    'candidates': {'variant,stages,kb': ms}}}."""
    return dict(_load()) if _state['cache_path'] else {}
