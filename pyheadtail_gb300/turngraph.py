"""Whole-turn CUDA graphs.

A PyHEADTAIL turn is a Python loop over elements; on the GPU each turn is
only a handful of kernels (fused track, slice merge, wake), so for small
bunches the host-side element code would dominate.  ``TurnGraph`` runs a
few turns eagerly through the normal ``track(beam)`` API, checks that the
turn's launch parameters have become stationary, captures one turn into a
CUDA graph and then replays it: one graph launch per turn, no host work.

Stationary means: constant energy (``p_increment == 0``; the reference's
p0 setter round trip settles after two turns), fixed or bunch-independent
cuts, and a wake history that no longer grows (single-turn wakes, or the
multi-turn ring already full -- the ring position is then advanced on the
device by capturing a full ring cycle).  While replaying, the host-side
Python objects (slice-set deques, ages) are not updated; the device state
(coordinates, moments ring, pending kicks) is.  After ``replay`` the beam
and elements can be used eagerly again.
"""
import ctypes

import torch

from . import _native as N


class _Recorder(object):
    """Logs the pointer-free parameters of every native call of a turn."""

    def __init__(self):
        self.log = []

    def __call__(self, name, args):
        sig = [name]
        for a in args:
            obj = getattr(a, '_obj', None)
            if isinstance(obj, N.Program):
                sig.append(bytes(obj))
            elif isinstance(obj, N.WakeSet):
                sig.append((obj.n_kicks,) + tuple(
                    (obj.kick[k].n_lags, obj.kick[k].factor)
                    for k in range(obj.n_kicks)))
            elif isinstance(obj, N.KickSet):
                sig.append((obj.n_kicks, bytes(obj.slicer)))
        self.log.append(tuple(sig))


class TurnGraph(object):
    """Capture / replay one turn of ``one_turn_map`` on ``beam``."""

    def __init__(self, one_turn_map, beam, warmup_turns=3):
        self.one_turn_map = list(one_turn_map)
        self.beam = beam
        self.warmup_turns = max(2, int(warmup_turns))
        self.graph = None
        self.turns_per_graph = 1

    def _eager_turn(self):
        for m in self.one_turn_map:
            m.track(self.beam)

    def _ring_cycle(self):
        """Turns per graph: the longest moment-ring of a WakeField, so that
        every replay leaves the ring position where it started."""
        n = 1
        for m in self.one_turn_map:
            st = getattr(m, '_state', None)
            if st is not None and st.n_ring > 1:
                n = max(n, st.n_ring)
        return n

    def _logged_turn(self):
        rec = _Recorder()
        N.RECORDERS.append(rec)
        try:
            self._eager_turn()
        finally:
            N.RECORDERS.remove(rec)
        return rec.log

    def capture(self, max_extra_turns=20):
        """Warm up eagerly (at least warmup_turns, then until two
        consecutive turns launch identical parameters), then capture."""
        prev = None
        for t in range(self.warmup_turns + max_extra_turns):
            log = self._logged_turn()
            if t + 1 >= self.warmup_turns and log == prev:
                break
            prev = log
        else:
            raise RuntimeError('turn parameters are not stationary (energy '
                               'ramp, bunch-dependent cuts or a growing wake '
                               'history); track eagerly instead')
        self.turns_per_graph = self._ring_cycle()
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(s):
            with torch.cuda.graph(g, stream=s):
                for _ in range(self.turns_per_graph):
                    self._eager_turn()
        torch.cuda.current_stream().wait_stream(s)
        self.graph = g
        return self

    def replay(self, n_graphs=1):
        """Run n_graphs * turns_per_graph turns."""
        if self.graph is None:
            self.capture()
        for _ in range(n_graphs):
            self.graph.replay()
        self.beam._engine.touch()


class StreamedTurns(object):
    """A stream of bunches, each copied in from host memory, tracked through
    its captured turn(s) and read out (its centroid), with the copy of one
    bunch overlapped with the turns of the previous one.

    ``make(slot)`` builds a (beam, one_turn_map) pair; ``n_slots`` of them
    (default 2) take the bunches in turn, each with its own captured
    TurnGraph.  ``push(host_coords)`` queues, on the slot's turn: the
    host-to-device copy of the six pinned host arrays into the slot's beam
    on a copy stream (after the slot's previous turn has finished with
    them), the graph replay on the compute stream (after the copy), a
    centroid pass (order-1 statistics of x and y) and the device-to-host
    copy of its record; it returns the centroid (x, y) of the bunch pushed
    ``n_slots`` calls earlier, or None.  ``drain()`` returns the rest.
    A beam state carries over in its slot (wake history, pending kick), as
    in an eager loop that reloads its coordinates."""

    def __init__(self, make, n_slots=2, warmup_turns=3):
        from .particles import statistics as S
        self._S = S
        self.slots = []
        for k in range(n_slots):
            beam, otm = make(k)
            tg = TurnGraph(otm, beam, warmup_turns=warmup_turns).capture()
            dev = beam._device
            self.slots.append(dict(
                beam=beam, tg=tg,
                rec=torch.zeros(S.RECORD_LEN, dtype=torch.float64, device=dev),
                host_rec=torch.zeros(S.RECORD_LEN,
                                     dtype=torch.float64).pin_memory(),
                copied=torch.cuda.Event(), done=torch.cuda.Event(),
                busy=False))
        self.copy_stream = torch.cuda.Stream()
        self.i = 0

    def _result(self, slot):
        slot['done'].synchronize()
        r = self._S.StatsRecord(slot['host_rec'].numpy().copy(), mask=0x5,
                                order=1)
        slot['busy'] = False
        return r.mean('x'), r.mean('y')

    def push(self, host_coords):
        slot = self.slots[self.i % len(self.slots)]
        self.i += 1
        out = self._result(slot) if slot['busy'] else None
        beam = slot['beam']
        cs = torch.cuda.current_stream()
        with torch.cuda.stream(self.copy_stream):
            self.copy_stream.wait_event(slot['done'])
            for k, t in host_coords.items():
                beam._c[k].copy_(t, non_blocking=True)
            slot['copied'].record(self.copy_stream)
        beam._engine.touch()
        cs.wait_event(slot['copied'])
        slot['tg'].replay(1)
        beam.launch_stats(slot['rec'], order=1, mask=0x5)
        slot['host_rec'].copy_(slot['rec'], non_blocking=True)
        slot['done'].record(cs)
        slot['busy'] = True
        return out

    def drain(self):
        out = []
        for k in range(len(self.slots)):
            slot = self.slots[(self.i + k) % len(self.slots)]
            if slot['busy']:
                out.append(self._result(slot))
        return out
