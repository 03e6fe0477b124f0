"""Batched form: many bunches of uneven sizes tracked by one persistent
launch per turn.

No counterpart in the reference, which tracks one bunch per ``track``
call.  A batch serves scans -- over chromaticity, intensity or wake
strength -- where every bunch has its own one-turn map but all share one
slicing.  Each bunch keeps behaving as a ``Particles`` (its coordinates
become views into the batch's arrays), and each bunch's element list is
the one a single-bunch user loop would run::

    batch = BunchBatch(bunches)
    turn = BatchedTurn(batch, [one_turn_map(b) for b in range(len(bunches))])
    turn.track(n_turns)          # eager turns, then CUDA-graph replay

Per turn, on the device (three launches whatever the number of bunches):
  1. ``phk_track_batch``: per work unit (a run of particles of one bunch),
     the bunch's pending wake kicks, its element program, binning and
     per-slice sums into the unit's partial column;
  2. ``phk_batch_finalize``: fixed-order merge of each bunch's columns into
     counts, centroids and the bunch's moment-ring slot;
  3. ``phk_wake_batch``: every bunch's multi-turn convolution -> its kick
     tables, applied in step 1 of the next turn.
On the host, the element programs are harvested per turn by running each
bunch's non-wake elements in deferred mode (their host scalars evolve
exactly as in the single-bunch loop).  Once the programs repeat and the
wake history is full, the turn is stationary and is captured as a CUDA
graph (one graph covers a full ring of the wake history).

The work units and launch shape (threads per CTA, particles per unit, CTAs
per SM) come from ``plan_units`` with a configuration that ``autotune``
picks by timing candidates on a scratch copy of the coordinates, cached in
a JSON file.
"""
import ctypes
import json
import math
import os

import numpy as np
import torch
from scipy.constants import c

from . import _engine as E
from . import _native as N
from .impedances.wakes import WakeField
from .impedances.wake_kicks import _SOURCE
from .particles.particles import COORDS

ALIGN = 4                       # bunch and unit starts: multiples of 4
THREADS = (128, 256, 512)
UNIT_TILES = (2, 4, 8, 16, 32)
DEFAULT_CONFIG = {'threads': 256, 'unit_tiles': 8, 'ctas_per_sm': 0}


def _vec(code):
    """Particles per thread of the batched kernel (FP64 and FP32 forms)."""
    return 2


# ------------------------------------------------------------ host planning

def bunch_offsets(counts, align=ALIGN):
    """Start of every bunch in the concatenated arrays (multiples of
    ``align``) and the total length."""
    off = np.zeros(len(counts), dtype=np.int64)
    pos = 0
    for b, n in enumerate(counts):
        off[b] = pos
        pos += (int(n) + align - 1) // align * align
    return off, int(pos)


def plan_units(offsets, counts, grid, unit_particles):
    """Split every bunch into units of at most ``unit_particles`` (a multiple
    of ALIGN) and give CTA g the contiguous unit range
    cta_first[g] .. cta_first[g+1]-1 holding about 1/grid of the particles.

    Returns dict(units: int64[n_units, 3] (start, end, bunch), column:
    int32[n_units], cta_first: int32[grid+1], bunch_columns: int32[nb+1],
    n_columns).  A CTA's consecutive units of one bunch share a column;
    columns are numbered in unit order, so those of bunch b are the range
    bunch_columns[b] .. bunch_columns[b+1]-1."""
    if unit_particles < ALIGN or unit_particles % ALIGN:
        raise ValueError('unit_particles must be a positive multiple of %d'
                         % ALIGN)
    nb = len(counts)
    units = []
    for b in range(nb):
        n = int(counts[b])
        for s in range(0, n, unit_particles):
            units.append((int(offsets[b]) + s,
                          int(offsets[b]) + min(s + unit_particles, n), b))
    units = np.array(units, dtype=np.int64).reshape(-1, 3)
    nu = len(units)
    sizes = units[:, 1] - units[:, 0] if nu else np.zeros(0, np.int64)
    total = int(sizes.sum())
    # cut the unit sequence where the running particle count crosses g/grid
    cta_first = np.zeros(grid + 1, dtype=np.int32)
    if nu:
        before = np.concatenate(([0], np.cumsum(sizes)[:-1]))
        targets = (np.arange(1, grid) * total) // grid
        cta_first[1:grid] = np.searchsorted(before, targets, side='left')
    cta_first[grid] = nu
    column = np.zeros(nu, dtype=np.int32)
    bunch_columns = np.zeros(nb + 1, dtype=np.int32)
    col = -1
    for g in range(grid):
        prev = -1
        for u in range(cta_first[g], cta_first[g + 1]):
            if units[u, 2] != prev:
                col += 1
                prev = units[u, 2]
            column[u] = col
    n_columns = col + 1
    # bunch b's columns: a contiguous range (units are in bunch order)
    firsts = np.full(nb, -1, dtype=np.int64)
    for u in range(nu - 1, -1, -1):
        firsts[units[u, 2]] = column[u]
    nxt = n_columns
    for b in range(nb - 1, -1, -1):
        if firsts[b] < 0:
            firsts[b] = nxt
        nxt = firsts[b]
    bunch_columns[:nb] = firsts
    bunch_columns[nb] = n_columns
    return dict(units=units, column=column, cta_first=cta_first,
                bunch_columns=bunch_columns, n_columns=max(n_columns, 1))


def unit_table(plan, device):
    """phk_unit array (start, end, bunch, column) as a device byte tensor."""
    u = plan['units']
    rec = np.zeros(len(u), dtype=[('start', '<i8'), ('end', '<i8'),
                                  ('bunch', '<i4'), ('column', '<i4')])
    if len(u):
        rec['start'], rec['end'], rec['bunch'] = u[:, 0], u[:, 1], u[:, 2]
        rec['column'] = plan['column']
    raw = np.frombuffer(rec.tobytes(), dtype=np.uint8).copy()
    if raw.size == 0:
        raw = np.zeros(24, dtype=np.uint8)
    return torch.from_numpy(raw).to(device)


def _to_device_bytes(structs, device):
    raw = b''.join(ctypes.string_at(ctypes.addressof(s), ctypes.sizeof(s))
                   for s in structs)
    return torch.from_numpy(np.frombuffer(raw, dtype=np.uint8).copy()).to(
        device)


# ------------------------------------------------------------ the batch

class BunchBatch(object):
    """Concatenates the coordinates of many bunches (same precision and
    device) into one set of six arrays; every bunch's coordinates become
    views into them, so each ``Particles`` keeps working on its own.
    Bunch b owns elements [offsets[b], offsets[b] + counts[b])."""

    def __init__(self, bunches):
        if not bunches:
            raise ValueError('a batch needs at least one bunch')
        b0 = bunches[0]
        for b in bunches:
            if b._code != b0._code or b._device != b0._device:
                raise ValueError('all bunches of a batch share precision and '
                                 'device')
            if set(COORDS) - set(b._c):
                raise ValueError('every bunch needs all six coordinates')
            b._engine.flush()
        self.bunches = list(bunches)
        self.code, self.device = b0._code, b0._device
        self.counts = np.array([b.macroparticlenumber for b in bunches],
                               dtype=np.int64)
        self.offsets, self.total = bunch_offsets(self.counts)
        dt = E.torch_dtype(self.code)
        self.storage = {}
        for q in COORDS:
            st = torch.zeros(max(self.total, ALIGN), dtype=dt,
                             device=self.device)
            for b, bunch in enumerate(bunches):
                o, n = int(self.offsets[b]), int(self.counts[b])
                st[o:o + n].copy_(bunch._c[q])
            self.storage[q] = st
        self._rebinds_seen = None
        for b, bunch in enumerate(bunches):
            o, n = int(self.offsets[b]), int(self.counts[b])
            for q in COORDS:
                bunch._c[q] = self.storage[q][o:o + n]
            bunch._engine.z_version += 1

    def __len__(self):
        return len(self.bunches)

    def check_views(self):
        """Raise if a bunch's coordinates were rebound away from the batch
        (e.g. ``bunch.x = new_array``).  Only bunches whose arrays were
        replaced since the last check are looked at."""
        now = [bunch._rebinds for bunch in self.bunches]
        if now == self._rebinds_seen:
            return
        for b, bunch in enumerate(self.bunches):
            o = int(self.offsets[b])
            for q in COORDS:
                t = bunch._c[q]
                if t.data_ptr() != self.storage[q][o:].data_ptr():
                    raise RuntimeError('bunch %d: coordinate %s no longer '
                                       'lives in the batch' % (b, q))
        self._rebinds_seen = now

    def coords_struct(self, storage=None):
        st = self.storage if storage is None else storage
        cs = N.Coords()
        cs.x, cs.xp = st['x'].data_ptr(), st['xp'].data_ptr()
        cs.y, cs.yp = st['y'].data_ptr(), st['yp'].data_ptr()
        cs.z, cs.dp = st['z'].data_ptr(), st['dp'].data_ptr()
        cs.n = self.total
        cs.dtype = self.code
        return cs


# ------------------------------------------------------------ autotuning

def _cache_key(batch, S, nk, programs):
    name = torch.cuda.get_device_name(batch.device)
    kinds = sorted({tuple(p.op[i].kind for i in range(p.n_ops))
                    for p in programs})
    return '|'.join([name, 'f64' if batch.code == N.PHK_F64 else 'f32',
                     'S%d' % S, 'k%d' % nk, 'nb%d' % len(batch),
                     'n2^%d' % int(round(math.log2(max(batch.total, 1)))),
                     repr(kinds)])


def default_cache_path():
    return os.path.join(os.path.dirname(os.path.abspath(__file__)),
                        '_build', 'autotune.json')


def load_cache(path):
    if path and os.path.exists(path):
        with open(path) as f:
            return json.load(f)
    return {}


def store_cache(path, cache):
    if not path:
        return
    os.makedirs(os.path.dirname(path), exist_ok=True)
    tmp = path + '.tmp'
    with open(tmp, 'w') as f:
        json.dump(cache, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def candidates(sm, max_grid):
    """Launch shapes to try: threads x particles per unit x CTAs per SM
    (``max_grid(threads)``: resident CTAs of the device, ``sm``: SMs)."""
    out = []
    for t in THREADS:
        g = max_grid(t)
        if g < 1:
            continue
        per_sm = max(1, g // sm)
        for ut in UNIT_TILES:
            for cps in sorted({1, max(1, per_sm // 2), per_sm}):
                out.append({'threads': t, 'unit_tiles': ut,
                            'ctas_per_sm': cps})
    return out


# ------------------------------------------------------------ the turn

class BatchedTurn(object):
    """One-turn maps of every bunch of a batch, run as three launches per
    turn (see module docstring).

    ``one_turn_maps[b]`` is bunch b's element list: transverse segments,
    longitudinal map and at most one ``WakeField`` (its own instance per
    bunch, fixed ``z_cuts``, the same slicing and kick types in every
    bunch).  ``config``: dict(threads, unit_tiles, ctas_per_sm) or None for
    the cached / default shape; ``autotune=True`` times the candidates."""

    def __init__(self, batch, one_turn_maps, config=None, autotune=False,
                 cache_path=None, warmup_turns=2):
        if len(one_turn_maps) != len(batch):
            raise ValueError('one element list per bunch')
        self.batch = batch
        self.maps, self.wakes = [], []
        for elements in one_turn_maps:
            ws = [e for e in elements if isinstance(e, WakeField)]
            if len(ws) > 1:
                raise ValueError('at most one WakeField per bunch')
            if ws and elements[-1] is not ws[0]:
                raise ValueError('the WakeField must be the last element')
            self.maps.append([e for e in elements
                              if not isinstance(e, WakeField)])
            self.wakes.append(ws[0] if ws else None)
        self._check_wakes()
        self.warmup_turns = warmup_turns
        self.turn = 0
        # optional list; when set, eager turns record (start, end) CUDA
        # events around the batched track launch, after calling
        # before_track() if given (e.g. to evict caches when timing)
        self.track_events = None
        self.before_track = None
        self.cache_path = (default_cache_path() if cache_path is None
                           else cache_path)
        self._graph = None
        self._last_programs = None
        self._allocate()
        progs = self._harvest()
        self._set_programs(progs)
        if config is None:
            key = _cache_key(batch, self.S, self.nk, progs)
            cached = load_cache(self.cache_path).get(key)
            if autotune:
                config = self.autotune(progs)
            elif cached is not None:
                config = cached
            else:
                config = dict(DEFAULT_CONFIG)
        self.config = config
        self._plan(config)
        self._pending_programs = progs

    # -- set-up
    def _check_wakes(self):
        ws = self.wakes
        if all(w is None for w in ws):
            self.S, self.nk, self.R = 1, 0, 1
            self.slicer = None
            return
        if any(w is None for w in ws):
            raise ValueError('either every bunch has a WakeField or none')
        if len({id(w) for w in ws}) != len(ws):
            raise ValueError('every bunch needs its own WakeField instance '
                             '(a WakeField keeps its bunch\'s history)')
        s0 = ws[0].slicer
        sig = None
        for w in ws:
            cfg = w.slicer.config
            if cfg[0] != 'uniform_bin' or cfg[2] or not cfg[3]:
                raise ValueError('batched wakes need a UniformBinSlicer with '
                                 'fixed z_cuts')
            if cfg != s0.config:
                raise ValueError('all bunches share one slicing')
            s = [(type(k).__name__, k.n_turns_wake, k._dense)
                 for k in w.wake_kicks]
            if sig is None:
                sig = s
            elif s != sig:
                raise ValueError('all bunches need the same wake kick types')
        if any(d for _, _, d in sig):
            raise ValueError('batched wakes use the convolution path')
        self.slicer = s0
        self.S = s0.n_slices
        self.nk = len(sig)
        self.R = ws[0].slice_set_deque.maxlen or 1

    def _allocate(self):
        bt, dev = self.batch, self.batch.device
        nb, S = len(bt), self.S
        dt = E.torch_dtype(bt.code)
        self.counts = torch.zeros(nb, S, dtype=torch.int32, device=dev)
        self.mean_x = torch.zeros(nb, S, dtype=torch.float64, device=dev)
        self.mean_y = torch.zeros(nb, S, dtype=torch.float64, device=dev)
        self.ring = torch.zeros(nb, self.R, 3, S, dtype=torch.float64,
                                device=dev)
        self.kicks = torch.zeros(nb, max(self.nk, 1), S, dtype=dt, device=dev)
        self._pk_cache = None     # PendingKicks naming rows of self.kicks
        self.status = torch.zeros(1, dtype=torch.int32, device=dev)
        if self.slicer is not None:
            b0 = bt.bunches[0]
            tail, head = self.slicer.get_long_cuts(b0)
            self.dslicer = self.slicer.device_slicer(tail, head, b0)
            self.z_bins = self.slicer.z_bins(tail, head)

    def _harvest(self):
        """Programs of this turn: each bunch's non-wake elements run in
        deferred mode; their ops are packed, not executed."""
        progs = []
        for bunch, elements in zip(self.batch.bunches, self.maps):
            eng = bunch._engine
            if not eng.idle:
                eng.flush()
            n0 = eng.launches
            for e in elements:
                e.track(bunch)
            if eng.launches != n0 or eng.kick is not None:
                raise ValueError('a batched one-turn map must fit one '
                                 'program (%d ops, %d detuners)'
                                 % (N.PHK_MAX_OPS, N.PHK_MAX_DETUNERS))
            progs.append(eng.program_struct(eng.ops))
            eng.ops = []
        return progs

    def _set_programs(self, progs):
        self.programs_host = (N.Program * len(progs))(*progs)
        self.programs_dev = _to_device_bytes(progs, self.batch.device)
        self._prog_bytes = ctypes.string_at(
            ctypes.addressof(self.programs_host),
            ctypes.sizeof(self.programs_host))

    def _plan(self, config, storage=None):
        bt = self.batch
        threads = int(config['threads'])
        tile = threads * _vec(bt.code)
        unit = int(config['unit_tiles']) * tile
        max_g = N.call('phk_batch_max_grid', bt.code, threads, self.S,
                       self.nk)
        sm = torch.cuda.get_device_properties(bt.device).multi_processor_count
        cps = int(config.get('ctas_per_sm', 0))
        grid = max_g if cps <= 0 else min(max_g, cps * sm)
        plan = plan_units(bt.offsets, bt.counts, grid, unit)
        dev = bt.device
        p = {'threads': threads, 'grid': grid, 'plan': plan,
             'units': unit_table(plan, dev),
             'cta_first': torch.from_numpy(plan['cta_first']).to(dev),
             'bunch_columns': torch.from_numpy(plan['bunch_columns']).to(dev),
             'partials': torch.zeros(3 * self.S * plan['n_columns'],
                                     dtype=torch.float64, device=dev)}
        if storage is None:
            self._p = p
        return p

    # -- structs
    def _batch_struct(self, p):
        b = N.Batch()
        b.n_bunches = len(self.batch)
        b.n_units = len(p['plan']['units'])
        b.n_columns = p['plan']['n_columns']
        b.grid = p['grid']
        b.threads = p['threads']
        b.units = p['units'].data_ptr()
        b.cta_first = p['cta_first'].data_ptr()
        b.programs = self.programs_dev.data_ptr()
        b.programs_host = ctypes.cast(self.programs_host,
                                      ctypes.POINTER(N.Program))
        b.kicks = self.kicks.data_ptr()
        b.status = self.status.data_ptr()
        return b

    def _accum(self, p):
        if self.slicer is None:
            return None
        a = N.Accum()
        a.slicer = self.dslicer.struct
        a.partials = p['partials'].data_ptr()
        a.partials_len = p['partials'].numel()
        a.grid = p['plan']['n_columns']
        return a

    def _kick_set(self):
        if self.nk == 0:
            return None
        ks = N.KickSet()
        ks.slicer = self.dslicer.struct
        ks.n_kicks = self.nk
        for k, kick in enumerate(self.wakes[0].wake_kicks):
            e = kick.pending_entry(self.kicks[0, k])
            ks.target[k] = e[0]
            ks.quad[k] = -1 if e[1] is None else e[1]
            ks.kick[k] = 0
        return ks

    def _wake_sets(self, head, n_lags_turns):
        """Device array of one phk_wake_set per bunch for ring slot
        ``head`` with ``n_lags_turns`` stored turns."""
        sets = []
        for b, (bunch, w) in enumerate(zip(self.batch.bunches, self.wakes)):
            times = self.slicer.times(self.z_bins, bunch.beta)
            ages = self._ages[:n_lags_turns]
            ws = N.WakeSet()
            ws.n_slices = self.S
            ws.ring_len = self.R
            ws.head = head
            ws.n_kicks = self.nk
            ws.out_dtype = self.batch.code
            ws.moments = self.ring[b].data_ptr()
            for k, kick in enumerate(w.wake_kicks):
                st = ws.kick[k]
                st.n_lags = kick._sync_tables([times] * len(ages), ages,
                                              [bunch.beta] * len(ages),
                                              self.S, self.ring.device)
                st.source = _SOURCE[kick.moment]
                st.dense = 0
                st.factor = float(kick._wake_factor(bunch))
                st.table = kick._table.data_ptr()
                st.out = self.kicks[b, k].data_ptr()
            sets.append(ws)
        return _to_device_bytes(sets, self.batch.device)

    # -- one turn
    def _launch_turn(self, p, coords, sets_dev, head, with_kicks,
                     wake=True):
        stream = E.stream_handle()
        b = self._batch_struct(p)
        acc = self._accum(p)
        ks = self._kick_set() if with_kicks else None
        ev = None
        if self.track_events is not None:
            if self.before_track is not None:
                self.before_track()
            ev = (torch.cuda.Event(enable_timing=True),
                  torch.cuda.Event(enable_timing=True))
            ev[0].record()
        N.call('phk_track_batch', ctypes.byref(b), ctypes.byref(coords),
               ctypes.byref(ks) if ks is not None else None,
               ctypes.byref(acc) if acc is not None else None, stream)
        if ev is not None:
            ev[1].record()
            self.track_events.append(ev)
        if acc is None or not wake:
            return
        ring_slot = self.ring[:, head]
        N.call('phk_batch_finalize', ctypes.byref(acc), len(self.batch),
               p['bunch_columns'].data_ptr(), self.counts.data_ptr(),
               self.mean_x.data_ptr(), self.mean_y.data_ptr(),
               ring_slot.data_ptr(), self.R * 3 * self.S, stream)
        if self.nk:
            N.call('phk_wake_batch', sets_dev.data_ptr(), len(self.batch),
                   self.S, self.nk, stream)

    def _eager_turn(self):
        progs = self._pending_programs
        if progs is None:
            progs = self._harvest()
        self._pending_programs = None
        self._set_programs(progs)
        head = self.turn % self.R
        n_turns_stored = min(self.turn + 1, self.R)
        self._advance_ages()
        sets = self._wake_sets(head, n_turns_stored) if self.nk else None
        self._sets_keep = sets
        self._launch_turn(self._p, self.batch.coords_struct(), sets, head,
                          with_kicks=self.turn > 0 and self.nk > 0)
        self.turn += 1
        stationary = (self._last_programs == self._prog_bytes)
        self._last_programs = self._prog_bytes
        return stationary

    def _advance_ages(self):
        """Ages of the stored turns as WakeField.track accumulates them
        (wakes.py:135-137): every stored age += C / (beta c), then the new
        turn enters at age 0."""
        if self.slicer is None:
            return
        if not hasattr(self, '_ages'):
            self._ages = []
        b0 = self.batch.bunches[0]
        d = b0.circumference / (b0.beta * c)
        self._ages = [0.] + [a + d for a in self._ages][:self.R - 1]

    def _capture(self):
        """CUDA graph of R turns (one full ring of the wake history)."""
        self._sets_per_head = []
        ages = list(self._ages)
        for r in range(self.R):
            head = (self.turn + r) % self.R
            self._sets_per_head.append(
                self._wake_sets(head, self.R) if self.nk else None)
        self._ages = ages
        coords = self.batch.coords_struct()
        s = torch.cuda.Stream(device=self.batch.device)
        s.wait_stream(torch.cuda.current_stream())
        g = torch.cuda.CUDAGraph()
        n0 = N.launch_count()
        with torch.cuda.graph(g, stream=s):
            for r in range(self.R):
                head = (self.turn + r) % self.R
                self._launch_turn(self._p, coords, self._sets_per_head[r],
                                  head, with_kicks=self.nk > 0)
        torch.cuda.current_stream().wait_stream(s)
        # library kernels captured per turn (one graph holds R turns)
        self.kernels_per_turn = (N.launch_count() - n0) // self.R
        self._graph = g
        self._graph_programs = self.programs_dev    # captured by pointer

    def _take_back_kicks(self):
        """The last turn's kicks were left pending on each bunch (so that
        reading a bunch's coordinates applies them, as in the single-bunch
        loop).  Take them back for the batched pass; a bunch whose kicks a
        read has already applied gets zero tables (adding 0.0 is exact)."""
        if self.nk == 0 or self.turn == 0:
            return
        for b, bunch in enumerate(self.batch.bunches):
            eng = bunch._engine
            if eng.ops:
                raise RuntimeError('bunch %d has pending element ops outside '
                                   'the batch' % b)
            eng.touch()
            if eng.kick is getattr(self, '_left', {}).get(b):
                eng.kick = None
            else:
                if eng.kick is not None:
                    eng.flush()
                self.kicks[b].zero_()

    def _leave_kicks(self):
        # one PendingKick per bunch, made once: it only names the bunch's
        # rows of the kick tables, which stay the same arrays
        if self._pk_cache is None and self.nk:
            self._pk_cache = [
                E.PendingKick(self.dslicer, [
                    kick.pending_entry(self.kicks[b, k])
                    for k, kick in enumerate(self.wakes[b].wake_kicks)])
                for b in range(len(self.batch.bunches))]
        self._left = {}
        for b, bunch in enumerate(self.batch.bunches):
            eng = bunch._engine
            eng.z_version += 1
            eng.touch()
            if self.nk == 0:
                continue
            pk = self._pk_cache[b]
            eng.kick = pk
            self._left[b] = pk

    def track(self, n_turns=1):
        """Advance every bunch by ``n_turns`` turns."""
        self.batch.check_views()
        self._take_back_kicks()
        try:
            self._track(n_turns)
        finally:
            self._leave_kicks()

    def _track(self, n_turns):
        done = 0
        while done < n_turns:
            if self._graph is not None and n_turns - done >= self.R:
                self._graph.replay()
                self.turn += self.R
                done += self.R
                continue
            stationary = self._eager_turn()
            done += 1
            if (self._graph is None and stationary and
                    self.turn >= max(self.warmup_turns, self.R) and
                    self.turn % self.R == 0):
                self._capture_after_eager()

    def _capture_after_eager(self):
        # the graph starts at ring slot self.turn % R with a full history
        self._capture()

    def eager_turns(self, n, before_each=None):
        """Run n turns without the graph (``before_each()`` is called
        before each, e.g. to evict caches when timing)."""
        self.batch.check_views()
        self._take_back_kicks()
        try:
            for _ in range(n):
                if before_each is not None:
                    before_each()
                self._eager_turn()
        finally:
            self._leave_kicks()

    def replay_turns(self, n):
        """Replay the captured graph n times (n * R turns)."""
        if self._graph is None:
            raise RuntimeError('no captured turn yet')
        self._take_back_kicks()
        try:
            for _ in range(n):
                self._graph.replay()
                self.turn += self.R
        finally:
            self._leave_kicks()

    def bunch_centroids(self):
        """Per-bunch x and y centroids of the particles inside the cuts at
        the last slicing, from the per-slice counts and means (device
        tensors of n_bunches entries)."""
        n = self.counts.to(torch.float64)
        tot = n.sum(dim=1).clamp(min=1)
        return ((n * self.mean_x).sum(dim=1) / tot,
                (n * self.mean_y).sum(dim=1) / tot)

    def read_status(self):
        """Device status word (0 ok, PHK_DEV_BAD_TABLE on a bad table)."""
        return int(self.status.item())

    # -- autotuning
    def autotune(self, progs=None, turns=3):
        """Time every candidate launch shape on a scratch copy of the
        coordinates and return (and cache) the fastest."""
        bt = self.batch
        scratch = {q: t.clone() for q, t in bt.storage.items()}
        coords = bt.coords_struct(scratch)
        max_grid = lambda t: N.call('phk_batch_max_grid', bt.code, t,
                                    self.S, self.nk)
        best, best_t = None, None
        sm = torch.cuda.get_device_properties(bt.device).multi_processor_count
        for cfg in candidates(sm, max_grid):
            p = self._plan(cfg, storage=scratch)
            b = self._batch_struct(p)
            acc = self._accum(p)
            ks = self._kick_set()
            times = []
            for it in range(turns + 1):
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record()
                N.call('phk_track_batch', ctypes.byref(b),
                       ctypes.byref(coords),
                       ctypes.byref(ks) if ks is not None else None,
                       ctypes.byref(acc) if acc is not None else None,
                       E.stream_handle())
                e1.record()
                torch.cuda.synchronize()
                if it:
                    times.append(e0.elapsed_time(e1))
            t = float(np.median(times))
            if best_t is None or t < best_t:
                best, best_t = cfg, t
        del scratch
        key = _cache_key(bt, self.S, self.nk,
                         progs if progs is not None else
                         list(self.programs_host))
        cache = load_cache(self.cache_path)
        cache[key] = best
        store_cache(self.cache_path, cache)
        self.tuned_ms = best_t
        return best
