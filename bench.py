#!/usr/bin/env python
"""Benchmark of the single-bunch turn loop on one GB300: macroparticle-turns/s.

Default workload (the configuration the target throughput is quoted on):
  multi-turn wake, 1e7 macroparticles, seed 2, matched 6D Gaussian (eps_n
  2.5 um, sigma_z 0.23 m, sigma_dp 1e-3), gamma 27.7, C = 6911.5 m, one
  transverse segment (Q 20.13 / 20.18, beta 50 m, Q' = 0), RF h = 4620,
  V = 4.5 MV, UniformBinSlicer 500 slices over (-0.69, 0.69) m, broadband
  resonator (10 MOhm/m, 1 GHz, Q = 1) plus a 50-turn resistive wall (20 mm,
  6911.5 m, 5.8e7 S/m).  The turn is [TransverseSegmentMap, RFSystems,
  WakeField]; a step is one replay of the turns captured as a CUDA graph
  (a full 50-turn cycle of the wake ring), repeated so that the timed
  region of each form lasts at least a second.

``value``  plain FP64 form (the drop-in), device time of the steps, inputs
           resident in HBM (240 / 480 MB, larger than L2; L2 is also
           flushed between steps).
``e2e``    the same turn(s) through the public API, wall clock: every step
           a bunch's coordinates copied from pinned host memory into a beam's
           arrays, one replay of its captured turn(s), its centroid record
           (order-1 statistics of x and y) copied back
           (``turngraph.StreamedTurns``: two beams take the steps in turn, so
           one step's copy overlaps the previous step's turn).
``forms``  the FP32 precision form measured the same way.
``--impl reference`` times the CPU oracle (a NumPy restatement of the
reference's turn loop, bit-identical to it on the golden fixtures) on the
same workload (the full bunch, one turn per step) on the host cores.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

C_RING = 6911.5038378975451
GAMMA = 27.7
Z_CUTS = (-0.69, 0.69)
ALPHA_C = 230. * 2 * np.pi * 0.017 / C_RING + GAMMA**-2
AMP = (1e-11, 1e-11, -5e-12)

WORKLOADS = {
    'c1': dict(n=100000, seed=0, slices=50, chroma=None, amp=None,
               longitudinal='linear', rw_turns=0,
               label='C1: 1e5 mp, linear maps, 50 slices, resonator'),
    'c2': dict(n=1000000, seed=1, slices=200, chroma=(5., 5.), amp=AMP,
               longitudinal='rf', rw_turns=0,
               label="C2: 1e6 mp, Q'=5, amplitude detuning, RF h=4620 "
                     "V=4.5MV, 200 slices, resonator"),
    'c3': dict(n=10000000, seed=2, slices=500, chroma=None, amp=None,
               longitudinal='rf', rw_turns=50,
               label='C3: 1e7 mp, 500 slices, resonator + 50-turn '
                     'resistive wall'),
    'c5': dict(n=50000000, seed=4, slices=1000, chroma=(2., 2.), amp=AMP,
               longitudinal='rf', rw_turns=50,
               label="C5: 5e7 mp, Q'=2, amplitude detuning, 1000 slices, "
                     'resonator + 50-turn resistive wall'),
}

# the batched workload: 256 bunches, sizes / chromaticities / intensities
# drawn with seed 3, 100 slices each, resonator wake, RF as C2
C4 = dict(n_bunches=256, seed=3, slices=100, chroma=(-5., 15.),
          intensity=(5e10, 2e11), log10_n=(4., 6.),
          label="C4: 256 bunches in one persistent launch, N_b log-uniform "
                "in [1e4, 1e6], own Q' in [-5, 15] and intensity in "
                "[5e10, 2e11], 100 slices each, resonator, RF h=4620")

L2_FLUSH_BYTES = 512 << 20
# shortest timed region of a form: steps are made of enough graph replays
MIN_TIMED_S = 1.0


def flush_l2(buf):
    """Evict the working set from L2 (untimed): write a buffer four times
    the L2 size, then read back its first half so that L2 ends up holding
    clean lines (otherwise the timed kernel would pay for writing back the
    flush buffer's dirty lines)."""
    buf.zero_()
    buf[:buf.numel() // 2].max()
# GPU spin (cycles) queued before each timed span, so that the span's events
# and kernels are all enqueued while the GPU is busy: the events then
# measure device time only, not the host's launch path
SPIN_CYCLES = 400000


def max_over_ranks(x, world):
    """Largest x over the ranks of the default process group (x itself for
    one rank).  Works with the NCCL (CUDA tensor) and gloo (CPU) backends."""
    if world <= 1:
        return float(x)
    import torch
    import torch.distributed as dist
    dev = 'cuda' if dist.get_backend() == 'nccl' else 'cpu'
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_value(units_per_step, ms_per_step_max, world):
    """Whole-job throughput of `world` replicas, each processing
    units_per_step per step, timed by the slowest rank."""
    return world * units_per_step / (ms_per_step_max * 1e-3)


def bench_config(w):
    """The workload as both arms report it (identical dicts)."""
    return {'workload': w['label'], 'n_macroparticles': w['n'],
            'n_slices': w['slices'],
            'wake': 'resonator' + (' + %d-turn resistive wall' % w['rw_turns']
                                   if w['rw_turns'] else ''),
            'l2': 'coordinates larger than L2; L2 flushed between steps '
                  '(untimed)'}


def bunch_coords(w):
    from pyheadtail_gb300.particles.generators import \
        gaussian_bunch_coordinates
    return gaussian_bunch_coordinates(w['n'], w['seed'], GAMMA, 2.5e-6, 2.5e-6,
                                      50., 50., 0.23, 1e-3)


def build_gpu(w, coords, precision):
    from scipy.constants import e, m_p
    from pyheadtail_gb300.general.printers import SilentPrinter
    from pyheadtail_gb300.impedances import wakes as W
    from pyheadtail_gb300.particles.particles import Particles
    from pyheadtail_gb300.particles.slicing import UniformBinSlicer
    from pyheadtail_gb300.trackers.detuners import (AmplitudeDetuning,
                                                    Chromaticity)
    from pyheadtail_gb300.trackers.longitudinal_tracking import (LinearMap,
                                                                 RFSystems)
    from pyheadtail_gb300.trackers.transverse_tracking import TransverseMap
    sp = SilentPrinter()
    # a shard of the bunch holds part of its particles at the bunch's
    # charge per macroparticle
    beam = Particles(len(coords['x']), 2.5e11 / w['n'], e, m_p, C_RING, GAMMA,
                     coords_n_momenta_dict=coords, precision=precision)
    dets = []
    if w['chroma']:
        dets.append(Chromaticity(*w['chroma']))
    if w['amp']:
        dets.append(AmplitudeDetuning(*w['amp']))
    z2 = np.zeros(2)
    tm = TransverseMap(np.array([0., C_RING]), z2, np.array([50., 50.]), z2,
                       z2, np.array([50., 50.]), z2, 20.13, 20.18, dets,
                       printer=sp)
    if w['longitudinal'] == 'rf':
        lm = RFSystems(C_RING, [4620], [4.5e6], [0.], [ALPHA_C], GAMMA,
                       charge=e, mass=m_p, printer=sp, warningprinter=sp)
    else:
        lm = LinearMap([ALPHA_C], C_RING, 0.017, printer=sp,
                       warningprinter=sp)
    sources = [W.CircularResonator(10e6, 1e9, 1.)]
    if w['rw_turns']:
        sources.append(W.CircularResistiveWall(0.02, C_RING, 5.8e7, 1e-12,
                                               n_turns_wake=w['rw_turns']))
    wf = W.WakeField(UniformBinSlicer(w['slices'], z_cuts=Z_CUTS,
                                      warningprinter=sp), *sources)
    return beam, list(tm) + [lm, wf]


def build_oracle(w, coords):
    from scipy.constants import e, m_p
    from oracle import turn_loop as T
    n = len(coords['x'])
    beam = T.Beam(coords, 2.5e11 / n, e, m_p, C_RING, GAMMA)
    z2 = np.zeros(2)
    segs = T.transverse_map([0., C_RING], z2, np.array([50., 50.]), z2, z2,
                            np.array([50., 50.]), z2, 20.13, 20.18,
                            chroma=w['chroma'], amplitude=w['amp'])
    if w['longitudinal'] == 'rf':
        lm = T.RFSystems(C_RING, [4620], [4.5e6], [0.], [ALPHA_C], GAMMA,
                         charge=e, mass=m_p)
    else:
        lm = T.LinearMap([ALPHA_C], C_RING, 0.017)
    sl = T.UniformBinSlicer(w['slices'], z_cuts=Z_CUTS)
    kicks = T.circular_resonator_kicks(sl, 10e6, 1e9, 1.)
    nmax = 1
    if w['rw_turns']:
        kicks += T.circular_resistive_wall_kicks(sl, 0.02, C_RING, 5.8e7,
                                                 1e-12, w['rw_turns'])
        nmax = w['rw_turns']
    return beam, list(segs) + [lm, T.WakeField(sl, kicks, nmax)]


# ------------------------------------------------------------------ clocks

class ClockSampler(object):
    """SM clock and clock-event reasons sampled every 10 ms during the timed
    region through NVML (read-only queries; no setting is changed), with
    nvidia-smi -lms 200 as the fallback when NVML cannot be loaded."""

    REASONS = {0x4: 'sw_power_cap', 0x8: 'hw_slowdown',
               0x20: 'sw_thermal_slowdown', 0x40: 'hw_thermal_slowdown',
               0x80: 'hw_power_brake_slowdown'}

    def __init__(self, device_index):
        self.dev = device_index
        self.samples = []
        self.max_mhz = None
        self._stop = threading.Event()
        self.t = None
        self.proc = None

    def _nvml(self):
        import ctypes
        lib = ctypes.CDLL('libnvidia-ml.so.1')
        if lib.nvmlInit_v2() != 0:
            raise OSError('nvmlInit failed')
        h = ctypes.c_void_p()
        if lib.nvmlDeviceGetHandleByIndex_v2(self.dev, ctypes.byref(h)) != 0:
            raise OSError('no NVML handle')
        mx = ctypes.c_uint()
        lib.nvmlDeviceGetMaxClockInfo(h, 1, ctypes.byref(mx))
        self.max_mhz = float(mx.value)
        reasons_fn = getattr(lib, 'nvmlDeviceGetCurrentClocksEventReasons',
                             None) or lib.nvmlDeviceGetCurrentClocksThrottleReasons
        return lib, h, reasons_fn

    def _loop_nvml(self, lib, h, reasons_fn):
        import ctypes
        clk = ctypes.c_uint()
        rs = ctypes.c_ulonglong()
        while not self._stop.is_set():
            if lib.nvmlDeviceGetClockInfo(h, 1, ctypes.byref(clk)) == 0 and \
                    reasons_fn(h, ctypes.byref(rs)) == 0:
                self.samples.append((float(clk.value), int(rs.value)))
            self._stop.wait(0.01)

    def start(self):
        try:
            lib, h, fn = self._nvml()
            self.t = threading.Thread(target=self._loop_nvml,
                                      args=(lib, h, fn), daemon=True)
            self.t.start()
            return
        except (OSError, AttributeError):
            pass
        try:
            self.proc = subprocess.Popen(
                ['nvidia-smi', '-i', str(self.dev),
                 '--query-gpu=clocks.sm,clocks.max.sm,'
                 'clocks_event_reasons.active', '--format=csv,noheader,nounits',
                 '-lms', '200'], stdout=subprocess.PIPE,
                stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._loop_smi, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _loop_smi(self):
        for line in self.proc.stdout:
            f = [x.strip() for x in line.split(',')]
            try:
                self.max_mhz = float(f[1])
                self.samples.append((float(f[0]), int(f[2], 16)))
            except (ValueError, IndexError):
                continue

    def stop(self):
        self._stop.set()
        if self.proc is not None:
            self.proc.terminate()
        if self.t is not None:
            self.t.join(timeout=5)
        if not self.samples:
            return None
        sm = [s[0] for s in self.samples]
        reasons = set()
        for _, r in self.samples:
            for bit, name in self.REASONS.items():
                if r & bit:
                    reasons.add(name)
        return {'sm_mhz': float(np.median(sm)), 'sm_max_mhz': self.max_mhz,
                'reasons': sorted(reasons), 'samples': len(sm),
                'source': 'nvml' if self.proc is None else 'nvidia-smi'}


# ------------------------------------------------------------------ GPU arm

def measured_peaks():
    p = os.path.join(ROOT, 'MEASURED_PEAKS.json')
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d['hbm_gbs']), 'measured'
    return 6800.0, 'fallback'


def profile_traffic(kernel_key):
    """DRAM bytes per particle of the track kernel from the committed ncu
    summary (profiles/traffic.json), or None."""
    p = os.path.join(ROOT, 'profiles', 'traffic.json')
    if not os.path.exists(p):
        return None
    with open(p) as f:
        d = json.load(f)
    return d.get(kernel_key)


def last_launch():
    """Kernel, ring stages and shared memory of the last fused pass."""
    import ctypes
    from pyheadtail_gb300 import _native as N
    v, s, m = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
    N.call('phk_last_track_launch', ctypes.byref(v), ctypes.byref(s),
           ctypes.byref(m))
    return {'kernel': 'phk::stream_kernel' if v.value == 1
            else 'phk::track_kernel', 'stages': s.value,
            'smem_bytes': m.value}


def time_form(w, coords, precision, steps, warmup, flush, tune=False):
    """Device time per turn (graph replay), track-kernel time, e2e.
    tune: time the launch plans of the FP32 pass first (its winner is
    the plan the turn is captured with)."""
    import tempfile
    from pyheadtail_gb300 import _native as N
    from pyheadtail_gb300 import tuning
    tune = tune and precision == 'fp32'
    if tune:
        tuning.enable(cache_path=os.path.join(tempfile.mkdtemp(),
                                              'plans.json'))
    try:
        return _time_form(w, coords, precision, steps, warmup, flush, tune)
    finally:
        if tune:
            tuning.enable(on=False)
            N.call('phk_set_track_plan', -1, -1, -1)


def _time_form(w, coords, precision, steps, warmup, flush, tune):
    import torch
    from pyheadtail_gb300 import _native as N
    from pyheadtail_gb300.turngraph import StreamedTurns, TurnGraph
    beam, elements = build_gpu(w, coords, precision)
    ring = max(1, w['rw_turns'])
    warm = max(warmup, ring + 2, 3)
    tg = TurnGraph(elements, beam, warmup_turns=warm).capture()
    tg.replay(1)                        # graph warm-up
    torch.cuda.synchronize()
    # replays per step, so that `steps` steps last at least MIN_TIMED_S
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(
        enable_timing=True)
    e0.record()
    tg.replay(1)
    e1.record()
    torch.cuda.synchronize()
    one = e0.elapsed_time(e1) * 1e-3
    reps = max(1, int(np.ceil(MIN_TIMED_S / (steps * one))))
    tpg = tg.turns_per_graph * reps
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    n0 = N.launch_count()
    for i in range(steps):
        flush_l2(flush)                 # evict L2 (outside the timed span)
        torch.cuda._sleep(SPIN_CYCLES)
        starts[i].record()
        tg.replay(reps)
        ends[i].record()
    torch.cuda.synchronize()
    graph_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    # the graph replays kernels captured through libphk: count them from
    # one eager turn (same sequence)
    for m in elements:                  # settle the pending-kick pipeline
        m.track(beam)
    n_eager0 = N.launch_count()
    for m in elements:
        m.track(beam)
    torch.cuda.synchronize()
    kernels_per_turn = N.launch_count() - n_eager0
    del n0
    # track kernel alone: eager turns with events around phk_track (the
    # last element, the WakeField, launches it)
    beam._engine.track_events = []
    for i in range(steps):
        for m in elements[:-1]:
            m.track(beam)
        flush_l2(flush)
        torch.cuda._sleep(SPIN_CYCLES)
        elements[-1].track(beam)
    torch.cuda.synchronize()
    evs = beam._engine.track_events
    beam._engine.track_events = None
    track_ms = [a.elapsed_time(b) for a, b in evs]
    launch = dict(last_launch(), tuned=tune)
    if tune:
        from pyheadtail_gb300 import tuning
        tuned = list(tuning.timings().values())
        launch['candidates_ms'] = tuned[0].get('candidates') if tuned else None
    # e2e: public API (turngraph.StreamedTurns), every step a bunch from
    # pinned host memory into a beam's coordinate arrays, one replay of its
    # captured turn(s), its centroid record read back; two beams take the
    # steps in turn, so a step's copy overlaps the previous step's turn
    host = {k: torch.from_numpy(np.ascontiguousarray(
        v.astype(np.float64 if precision == 'fp64' else np.float32))
    ).pin_memory() for k, v in coords.items()}
    h2d = sum(t.numel() * t.element_size() for t in host.values())
    tg_turns = tg.turns_per_graph
    del tg, beam, elements
    torch.cuda.empty_cache()
    st = StreamedTurns(lambda k: build_gpu(w, coords, precision), n_slots=2,
                       warmup_turns=warm)
    for _ in range(4):                   # loads torch's copy / event paths
        st.push(host)
    st.drain()
    # e2e steps are one graph replay each (a bunch in, its turns, a record
    # out), enough of them to last about MIN_TIMED_S
    n_e2e = max(4, int(np.ceil(MIN_TIMED_S / one)))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for i in range(n_e2e):
        st.push(host)
    cx, cy = st.drain()[-1]
    e2e_s = [(time.perf_counter() - t0) / n_e2e] * n_e2e
    del st
    torch.cuda.empty_cache()
    return dict(graph_ms=graph_ms, turns_per_step=tpg,
                e2e_turns_per_step=tg_turns, track_ms=track_ms,
                e2e_s=e2e_s, h2d=h2d, d2h=8 * 34,
                kernels_per_turn=kernels_per_turn, centroid=(cx, cy),
                launch=launch)


def host_cpu():
    """The host the CPU baseline ran on: architecture, CPU model (x86
    'model name', or the Arm implementer / part codes), logical CPUs and
    the thread settings of the numerical libraries.  Never raises."""
    import platform
    out = {'machine': platform.machine(), 'logical_cpus': os.cpu_count(),
           'OMP_NUM_THREADS': os.environ.get('OMP_NUM_THREADS'),
           'OPENBLAS_NUM_THREADS': os.environ.get('OPENBLAS_NUM_THREADS')}
    model = None
    try:
        fields = {}
        with open('/proc/cpuinfo') as f:
            for line in f:
                if ':' in line:
                    k, v = line.split(':', 1)
                    fields.setdefault(k.strip(), v.strip())
        if 'model name' in fields:
            model = fields['model name']
        elif 'CPU part' in fields:
            model = 'implementer %s part %s' % (
                fields.get('CPU implementer', '?'), fields['CPU part'])
    except (OSError, ValueError):
        pass
    out['model'] = model or platform.processor() or None
    return out


def cpu_baseline(w, coords, budget_s=12.0):
    """Oracle (NumPy restatement of the reference) on the host, 1 thread,
    on a bounded sample: the full bunch (up to 1e7 particles), turns until
    about budget_s of CPU time (at least one)."""
    n = len(coords['x'])
    ns = min(n, 10000000)
    sub = {k: v[:ns].copy() for k, v in coords.items()}
    beam, els = build_oracle(w, sub)
    for m in els:                       # one untimed turn
        m.track(beam)
    t0 = time.perf_counter()
    turns = 0
    while True:
        for m in els:
            m.track(beam)
        turns += 1
        if time.perf_counter() - t0 > budget_s or turns >= 200:
            break
    dt = time.perf_counter() - t0
    return {'value': ns * turns / dt, 'unit': 'macroparticle-turns/s',
            'cores': 1, 'kind': 'port', 'host': host_cpu(),
            'sample': '%d macroparticles x %d turns of the same workload '
                      '(oracle: NumPy restatement of the reference, single '
                      'thread, like the reference)' % (ns, turns)}


def run_eager(a):
    """A short run for profilers: `a.eager_turns` eager turns of the
    workload in each selected form (no graph, no timing loop), then the
    track-kernel time of the last three turns and the bunch centroid."""
    import tempfile
    import torch
    from pyheadtail_gb300 import tuning
    w = WORKLOADS[a.workload]
    coords = bunch_coords(w)
    for precision in ('fp64', 'fp32'):
        if a.form not in ('all', precision):
            continue
        if a.autotune and precision == 'fp32':
            tuning.enable(cache_path=os.path.join(tempfile.mkdtemp(),
                                                  'plans.json'))
        beam, elements = build_gpu(w, coords, precision)
        for t in range(a.eager_turns):
            if t == a.eager_turns - 3:
                beam._engine.track_events = []
            for m in elements[:-1]:
                m.track(beam)
            if t >= a.eager_turns - 3:
                # the GPU busy while the pass is launched: its events time
                # the device only
                torch.cuda._sleep(SPIN_CYCLES)
            elements[-1].track(beam)
        torch.cuda.synchronize()
        evs = beam._engine.track_events or []
        print(json.dumps({'form': precision, 'turns': a.eager_turns,
                          'track_ms': [x.elapsed_time(y) for x, y in evs],
                          'launch': last_launch(),
                          'tuning': tuning.timings()
                          if tuning.enabled() else None,
                          'mean_x': float(beam.mean_x())}))
        tuning.enable(on=False)
        del beam, elements
        torch.cuda.empty_cache()


def run_ours(a, rank, world):
    import torch
    w = WORKLOADS[a.workload]
    dev = rank % max(1, torch.cuda.device_count())
    torch.cuda.set_device(dev)
    coords = bunch_coords(w)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32,
                        device='cuda')
    hbm_peak, peak_kind = measured_peaks()
    sampler = ClockSampler(dev)
    forms = {}
    sampler.start()
    for precision in ('fp64', 'fp32'):
        if a.form not in ('all', precision):
            continue
        r = time_form(w, coords, precision, a.steps, a.warmup, flush,
                      tune=a.autotune)
        bytes_pp = 96 if precision == 'fp64' else 48
        step_ms = float(np.sum(r['graph_ms']))
        turns = a.steps * r['turns_per_step']
        track_avg = float(np.mean(r['track_ms']))
        achieved = bytes_pp * w['n'] / (track_avg * 1e-3) / 1e9
        tpp = profile_traffic('track_%s_%s' % (a.workload, precision))
        e2e_t = float(np.sum(r['e2e_s']))
        forms[precision] = {
            'value': w['n'] * turns / (step_ms * 1e-3),
            'ms_per_step': step_ms / a.steps,
            'turns_per_step': r['turns_per_step'],
            'kernels_per_turn': r['kernels_per_turn'],
            'launch_plan': r['launch'],
            'roofline': {'bound': 'hbm', 'achieved': achieved,
                         'peak': hbm_peak, 'unit': 'GB/s',
                         'frac': achieved / hbm_peak,
                         'peak_kind': peak_kind,
                         'traffic': None if tpp is None else tpp * w['n'],
                         'kernel': r['launch']['kernel'],
                         'kernel_ms': track_avg,
                         'algorithmic_bytes_per_launch': bytes_pp * w['n'],
                         'note': ('HBM fraction of a kernel bound by the FP64 '
                                  'pipe (GB300 runs FP64 at 1/59 of the FP32 '
                                  'rate); forms.fp32 is the HBM-bound form'
                                  if precision == 'fp64' else
                                  'HBM-bound form')},
            'e2e': {'value': w['n'] * r['e2e_turns_per_step'] *
                    len(r['e2e_s']) / e2e_t,
                    'unit': 'macroparticle-turns/s',
                    'h2d_bytes_per_step': r['h2d'],
                    'd2h_bytes_per_step': r['d2h']},
        }
    clocks = sampler.stop()
    head = forms.get('fp64') or forms['fp32']
    prec = 'fp64' if 'fp64' in forms else 'fp32'
    # multi-GPU: independent replicas, the slowest rank defines the time
    ms_max = max_over_ranks(head['ms_per_step'], world)
    if rank != 0:
        return
    out = {
        'metric': 'macroparticle-turns/s on 1 GB300: FP32/batched vs FP64 '
                  'plain; % HBM roofline',
        'value': job_value(w['n'] * head['turns_per_step'], ms_max, world),
        'unit': 'macroparticle-turns/s',
        'n_gpus': world, 'steps': a.steps, 'warmup': a.warmup,
        'ms_per_step': ms_max,
        'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None,
        'dtype': 'f64' if prec == 'fp64' else 'f32',
        'data': 'synthetic: seeded 6D Gaussian bunch (reference generator '
                'draw order), no dataset',
        'config': bench_config(w),
        'form': prec, 'turns_per_step': head['turns_per_step'],
        'timing': 'CUDA events around CUDA-graph replays of the turn; '
                  'inputs resident in HBM',
        'parallelism': 'replicas' if world > 1 else 'single GPU',
        'roofline': head['roofline'],
        'e2e': head['e2e'],
        'gpu_launches': head['kernels_per_turn'] * head['turns_per_step'] *
        a.steps,
        'clocks': clocks,
        'forms': forms,
    }
    if world == 1 and not a.no_cpu_baseline:
        out['cpu_baseline'] = cpu_baseline(w, coords)
    print(json.dumps(out))


# ------------------------------------------------------ sharded bunch arm

def run_sharded(a, rank, world):
    """One bunch split over the ranks by particles (pyheadtail_gb300.shards):
    every rank tracks its shard; the slice sums are all-gathered and
    merged in rank order every turn; the wake is computed on every rank.
    Eager turns (the all-gather is not captured in a graph); total work
    fixed as N grows (strong scaling)."""
    import torch
    from pyheadtail_gb300 import shards as SH
    w = WORKLOADS[a.workload]
    coords = bunch_coords(w)
    sh = SH.Shards()
    lo, hi = sh.range(w['n'])
    part = {k: np.ascontiguousarray(v[lo:hi]) for k, v in coords.items()}
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32,
                        device='cuda')
    sampler = ClockSampler(torch.cuda.current_device())
    forms = {}
    sampler.start()
    for precision in ('fp64', 'fp32'):
        if a.form not in ('all', precision):
            continue
        beam, elements = build_gpu(w, part, precision)
        SH.shard(beam, sh)
        for _ in range(max(a.warmup, w['rw_turns'] + 2, 3)):
            for m in elements:
                m.track(beam)
        torch.cuda.synchronize()
        ms = []
        for i in range(a.steps):
            flush_l2(flush)
            if world > 1:
                import torch.distributed as dist
                dist.barrier()
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            for m in elements:
                m.track(beam)
            e1.record()
            torch.cuda.synchronize()
            ms.append(e0.elapsed_time(e1))
        step = max_over_ranks(float(np.mean(ms)), world)
        forms[precision] = {'value': w['n'] / (step * 1e-3),
                            'ms_per_step': step, 'turns_per_step': 1,
                            'shard_macroparticles': hi - lo}
        del beam, elements
        torch.cuda.empty_cache()
    clocks = sampler.stop()
    if rank != 0:
        return
    prec = 'fp64' if 'fp64' in forms else 'fp32'
    head = forms[prec]
    print(json.dumps({
        'metric': 'macroparticle-turns/s of one bunch sharded over the '
                  'GPUs',
        'value': head['value'], 'unit': 'macroparticle-turns/s',
        'n_gpus': world, 'steps': a.steps, 'warmup': a.warmup,
        'ms_per_step': head['ms_per_step'], 'higher_is_better': True,
        'scaling': 'strong', 'vs_baseline': None,
        'dtype': 'f64' if prec == 'fp64' else 'f32',
        'data': 'synthetic: seeded 6D Gaussian bunch (reference generator '
                'draw order), no dataset',
        'config': bench_config(w), 'form': prec, 'turns_per_step': 1,
        'timing': 'CUDA events around eager turns, max over ranks; L2 '
                  'flushed between turns',
        'parallelism': 'sharded single bunch: particles split over %d '
                       'ranks, slice sums all-gathered and merged in rank '
                       'order every turn, wake replicated' % world,
        'clocks': clocks, 'forms': forms}))


# ------------------------------------------------------------ batched arm

def c4_draws():
    rs = np.random.RandomState(C4['seed'])
    nb = C4['n_bunches']
    sizes = np.round(10 ** rs.uniform(*C4['log10_n'], size=nb)).astype(
        np.int64)
    chroma = rs.uniform(*C4['chroma'], size=nb)
    intensity = rs.uniform(*C4['intensity'], size=nb)
    return sizes, chroma, intensity


def c4_coords(n, b, precision, device='cuda'):
    """Matched Gaussian bunch of n particles drawn on the device with a
    per-bunch seed (same sigmas as the single-bunch workloads)."""
    import torch
    g = torch.Generator(device=device).manual_seed(3000 + b)
    eps = 2.5e-6 / np.sqrt(GAMMA**2 - 1)
    sig = {'x': np.sqrt(eps * 50.), 'xp': np.sqrt(eps / 50.),
           'y': np.sqrt(eps * 50.), 'yp': np.sqrt(eps / 50.),
           'z': 0.23, 'dp': 1e-3}
    dt = torch.float64 if precision == 'fp64' else torch.float32
    return {k: (torch.randn(n, generator=g, device=device,
                            dtype=torch.float64) * s).to(dt)
            for k, s in sig.items()}


def c4_bunch(n, q, intensity, coords, precision):
    from scipy.constants import e, m_p
    from pyheadtail_gb300.general.printers import SilentPrinter
    from pyheadtail_gb300.impedances import wakes as W
    from pyheadtail_gb300.particles.particles import Particles
    from pyheadtail_gb300.particles.slicing import UniformBinSlicer
    from pyheadtail_gb300.trackers.detuners import Chromaticity
    from pyheadtail_gb300.trackers.longitudinal_tracking import RFSystems
    from pyheadtail_gb300.trackers.transverse_tracking import TransverseMap
    sp = SilentPrinter()
    beam = Particles(n, intensity / n, e, m_p, C_RING, GAMMA,
                     coords_n_momenta_dict=coords, precision=precision)
    z2 = np.zeros(2)
    tm = TransverseMap(np.array([0., C_RING]), z2, np.array([50., 50.]), z2,
                       z2, np.array([50., 50.]), z2, 20.13, 20.18,
                       [Chromaticity(q, q)], printer=sp)
    rf = RFSystems(C_RING, [4620], [4.5e6], [0.], [ALPHA_C], GAMMA,
                   charge=e, mass=m_p, printer=sp, warningprinter=sp)
    wf = W.WakeField(UniformBinSlicer(C4['slices'], z_cuts=Z_CUTS,
                                      warningprinter=sp),
                     W.CircularResonator(10e6, 1e9, 1.))
    return beam, list(tm) + [rf, wf]


def time_batch(precision, steps, warmup, flush, autotune, bunches=None):
    """bunches: indices of the train's bunches this rank tracks (all by
    default)."""
    import torch
    from pyheadtail_gb300 import _native as N
    from pyheadtail_gb300.batch import BatchedTurn, BunchBatch
    sizes, chroma, intensity = c4_draws()
    beams, maps = [], []
    for b in (range(len(sizes)) if bunches is None else bunches):
        c = c4_coords(int(sizes[b]), b, precision)
        beam, els = c4_bunch(int(sizes[b]), float(chroma[b]),
                             float(intensity[b]), c, precision)
        beams.append(beam)
        maps.append(els)
    batch = BunchBatch(beams)
    turn = BatchedTurn(batch, maps, autotune=autotune)
    turn.track(max(warmup, 3))           # eager warm-up, then capture
    for _ in range(20):
        if turn._graph is not None:
            break
        turn.track(1)
    if turn._graph is None:
        raise RuntimeError('batched turn did not become stationary')
    turn.track(1)
    torch.cuda.synchronize()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    for i in range(steps):
        flush_l2(flush)
        torch.cuda._sleep(SPIN_CYCLES)
        starts[i].record()
        turn.replay_turns(1)
        ends[i].record()
    torch.cuda.synchronize()
    graph_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    # library kernels in one captured turn
    kernels_per_turn = turn.kernels_per_turn
    del N
    # the batched track kernel alone: eager turns with events around it

    def spaced():
        flush_l2(flush)
        torch.cuda._sleep(SPIN_CYCLES)
    turn.track_events = []
    turn.before_track = spaced
    turn.eager_turns(steps)
    turn.before_track = None
    torch.cuda.synchronize()
    track_ms = [a.elapsed_time(b) for a, b in turn.track_events]
    turn.track_events = None
    # e2e: every bunch's coordinates from pinned host memory into the
    # batch, one turn, the per-bunch centroids read back
    host = {k: torch.empty(batch.total, dtype=batch.storage[k].dtype
                           ).pin_memory() for k in batch.storage}
    for k in host:
        host[k].copy_(batch.storage[k][:batch.total])
    h2d = sum(t.numel() * t.element_size() for t in host.values())
    e2e_s = []
    for i in range(max(3, steps // 2) + 1):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for k, t in host.items():
            batch.storage[k][:batch.total].copy_(t, non_blocking=True)
        turn.track(1)
        cx, cy = turn.bunch_centroids()
        res = torch.stack([cx, cy]).cpu()
        if i:                            # the first step loads torch's kernels
            e2e_s.append(time.perf_counter() - t0)
    return dict(graph_ms=graph_ms, track_ms=track_ms, e2e_s=e2e_s, h2d=h2d,
                d2h=res.numel() * 8, kernels_per_turn=kernels_per_turn,
                total=int(batch.total), particles=int(sizes.sum()),
                config=dict(turn.config), grid=turn._p['grid'],
                units=len(turn._p['plan']['units']),
                columns=turn._p['plan']['n_columns'])


def _c4_oracle_runs(worker, workers, cap=300000):
    """Oracle beams and elements of the batch's bunches worker, worker +
    workers, ... up to about cap particles."""
    from scipy.constants import e, m_p
    from oracle import turn_loop as T
    sizes, chroma, intensity = c4_draws()
    runs, tot = [], 0
    for b in range(worker, len(sizes), workers):
        n = int(sizes[b])
        if tot and tot + n > cap:
            continue
        rng = np.random.RandomState(3000 + b)
        eps = 2.5e-6 / np.sqrt(GAMMA**2 - 1)
        sig = {'x': np.sqrt(eps * 50.), 'xp': np.sqrt(eps / 50.),
               'y': np.sqrt(eps * 50.), 'yp': np.sqrt(eps / 50.),
               'z': 0.23, 'dp': 1e-3}
        coords = {k: rng.normal(0, s, n) for k, s in sig.items()}
        beam = T.Beam(coords, intensity[b] / n, e, m_p, C_RING, GAMMA)
        z2 = np.zeros(2)
        segs = T.transverse_map([0., C_RING], z2, np.array([50., 50.]), z2,
                                z2, np.array([50., 50.]), z2, 20.13, 20.18,
                                chroma=(chroma[b], chroma[b]), amplitude=None)
        lm = T.RFSystems(C_RING, [4620], [4.5e6], [0.], [ALPHA_C], GAMMA,
                         charge=e, mass=m_p)
        sl = T.UniformBinSlicer(C4['slices'], z_cuts=Z_CUTS)
        wf = T.WakeField(sl, T.circular_resonator_kicks(sl, 10e6, 1e9, 1.), 1)
        runs.append((beam, list(segs) + [lm, wf]))
        tot += n
        if tot >= cap:
            break
    return runs, tot


def _c4_oracle_worker(args):
    """One process of the CPU baseline: its bunches, one warm-up turn, then
    turns until about budget_s.  Returns (particles, turns, seconds,
    bunches)."""
    worker, workers, budget_s = args
    runs, tot = _c4_oracle_runs(worker, workers)
    for beam, els in runs:
        for m in els:
            m.track(beam)
    t0 = time.perf_counter()
    turns = 0
    while True:
        for beam, els in runs:
            for m in els:
                m.track(beam)
        turns += 1
        if time.perf_counter() - t0 > budget_s or turns >= 200:
            break
    return tot, turns, time.perf_counter() - t0, len(runs)


def c4_oracle_sample(budget_s=12.0, procs=None):
    """The oracle on a bounded sample of the batch, one process per host
    core: the bunches are independent, so each process tracks its own
    bunches (about 3e5 particles) as the reference would run them side by
    side.  Returns (macroparticle-turns/s summed over the processes over
    the longest process's time, particles, turns of the slowest process,
    bunches, processes).  Processes are spawned, not forked: the caller
    may already hold a CUDA context."""
    P = procs or os.cpu_count() or 1
    if P <= 1:
        tot, turns, dt, nbs = _c4_oracle_worker((0, 1, budget_s))
        return tot * turns / dt, tot, turns, nbs, 1
    import multiprocessing
    ctx = multiprocessing.get_context('spawn')
    with ctx.Pool(P) as pool:
        res = pool.map(_c4_oracle_worker,
                       [(w, P, budget_s) for w in range(P)])
    wall = max(r[2] for r in res)
    work = sum(r[0] * r[1] for r in res)
    return (work / wall, sum(r[0] for r in res), min(r[1] for r in res),
            sum(r[3] for r in res), P)


def run_batch(a, rank, world):
    import torch
    dev = rank % max(1, torch.cuda.device_count())
    torch.cuda.set_device(dev)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32,
                        device='cuda')
    hbm_peak, peak_kind = measured_peaks()
    steps = a.steps if a.steps_given else 50
    sampler = ClockSampler(dev)
    forms = {}
    sampler.start()
    bunches = None
    if a.shard:
        # the train's bunches packed over the ranks (whole bunches, no
        # exchange)
        from pyheadtail_gb300.shards import pack_bunches
        bunches = pack_bunches(c4_draws()[0], world)[rank]
    for precision in ('fp32', 'fp64'):
        if a.form not in ('all', precision):
            continue
        r = time_batch(precision, steps, a.warmup, flush, a.autotune,
                       bunches)
        bytes_pp = 96 if precision == 'fp64' else 48
        n = r['particles']
        step_ms = float(np.sum(r['graph_ms']))
        track_avg = float(np.mean(r['track_ms']))
        achieved = bytes_pp * n / (track_avg * 1e-3) / 1e9
        tpp = profile_traffic('track_batch_c4_%s' % precision)
        e2e_t = float(np.sum(r['e2e_s']))
        forms[precision] = {
            'value': n * steps / (step_ms * 1e-3),
            'ms_per_step': step_ms / steps,
            'kernels_per_turn': r['kernels_per_turn'],
            'launch': {'config': r['config'], 'grid': r['grid'],
                       'units': r['units'], 'columns': r['columns']},
            'roofline': {'bound': 'hbm', 'achieved': achieved,
                         'peak': hbm_peak, 'unit': 'GB/s',
                         'frac': achieved / hbm_peak, 'peak_kind': peak_kind,
                         'traffic': None if tpp is None else tpp * n,
                         'kernel': 'phk::batch_track_kernel',
                         'kernel_ms': track_avg,
                         'algorithmic_bytes_per_launch': bytes_pp * n},
            'e2e': {'value': n * len(r['e2e_s']) / e2e_t,
                    'unit': 'macroparticle-turns/s',
                    'h2d_bytes_per_step': r['h2d'],
                    'd2h_bytes_per_step': r['d2h']},
            'particles': n,
        }
    clocks = sampler.stop()
    prec = 'fp32' if 'fp32' in forms else 'fp64'
    head = forms[prec]
    ms_max = max_over_ranks(head['ms_per_step'], world)
    total = head['particles']
    if a.shard:
        total = int(c4_draws()[0].sum())
    if rank != 0:
        return
    out = {
        'metric': 'macroparticle-turns/s on 1 GB300: FP32/batched vs FP64 '
                  'plain; % HBM roofline',
        'value': (total / (ms_max * 1e-3) if a.shard else
                  job_value(head['particles'], ms_max, world)),
        'unit': 'macroparticle-turns/s',
        'n_gpus': world, 'steps': steps, 'warmup': a.warmup,
        'ms_per_step': ms_max,
        'higher_is_better': True,
        'scaling': 'strong' if a.shard else 'weak', 'vs_baseline': None,
        'dtype': 'f32' if prec == 'fp32' else 'f64',
        'data': 'synthetic: 256 seeded matched Gaussian bunches drawn on the '
                'device, no dataset',
        'config': {'workload': C4['label'],
                   'n_macroparticles': total,
                   'n_bunches': C4['n_bunches'], 'n_slices': C4['slices'],
                   'form': 'batched ' + prec, 'turns_per_step': 1,
                   'l2': 'flushed between steps (512 MiB write + 256 MiB '
                         'read-back, untimed); working set larger than L2',
                   'timing': 'CUDA events around a CUDA-graph replay of the '
                             'batched turn; inputs resident in HBM',
                   'parallelism': ('bunches packed over %d ranks' % world
                                   if a.shard else
                                   'replicas' if world > 1 else 'single GPU')},
        'roofline': head['roofline'],
        'e2e': head['e2e'],
        'gpu_launches': head['kernels_per_turn'] * steps,
        'clocks': clocks,
        'forms': forms,
    }
    if world == 1 and not a.no_cpu_baseline:
        v, tot, turns, nbs, procs = c4_oracle_sample()
        out['cpu_baseline'] = {
            'value': v, 'unit': 'macroparticle-turns/s', 'cores': procs,
            'kind': 'port', 'host': host_cpu(),
            'sample': '%d macroparticles (%d bunches of the batch, one '
                      'process per core) x >= %d turns (oracle)'
                      % (tot, nbs, turns)}
    print(json.dumps(out))


def run_reference_c4(a, rank, world):
    if rank != 0:
        return
    t0 = time.perf_counter()
    v, tot, turns, nbs, procs = c4_oracle_sample(
        budget_s=max(2.0, 0.2 * a.steps))
    del t0
    sample = ('%d macroparticles (%d bunches of the batch, one process per '
              'core) x >= %d turns' % (tot, nbs, turns))
    print(json.dumps({
        'impl': 'reference',
        'metric': 'macroparticle-turns/s on 1 GB300: FP32/batched vs FP64 '
                  'plain; % HBM roofline',
        'value': v, 'unit': 'macroparticle-turns/s', 'n_gpus': world,
        'steps': a.steps, 'warmup': a.warmup,
        'ms_per_step': tot / v * 1e3, 'higher_is_better': True,
        'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f64',
        'data': 'synthetic: seeded matched Gaussian bunches',
        'config': {'workload': C4['label'], 'n_bunches': C4['n_bunches'],
                   'n_slices': C4['slices'], 'form': 'fp64'},
        'cpu_baseline': {'value': v, 'unit': 'macroparticle-turns/s',
                         'cores': procs, 'kind': 'port', 'sample': sample,
                         'host': host_cpu()},
        'e2e': {'value': v, 'unit': 'macroparticle-turns/s',
                'h2d_bytes_per_step': 0, 'd2h_bytes_per_step': 0},
    }))


# ------------------------------------------------------------ statistics pass

def run_stats_pass(a, rank, world):
    """Time the bunch statistics pass (Particles.launch_stats ->
    phk_bunch_stats) on the workload's bunch size with random coordinates
    made on the device: centroids of x and y (order 1), centroids of all
    six coordinates, and the order-2 pass behind sigma / emittance / Twiss.
    Prints one JSON line; not the headline metric."""
    import torch
    from pyheadtail_gb300.particles.particles import Particles
    from scipy.constants import e, m_p
    if rank != 0:
        return
    w = WORKLOADS[a.workload]
    n = w['n']
    peak, peak_kind = measured_peaks()
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32,
                        device='cuda')
    cases = {}
    for prec in ('fp32', 'fp64'):
        if a.form not in ('all', prec):
            continue
        dt = torch.float32 if prec == 'fp32' else torch.float64
        g = torch.Generator(device='cuda').manual_seed(w['seed'])
        coords = {q: 1e-3 * torch.randn(n, dtype=dt, device='cuda',
                                        generator=g)
                  for q in ('x', 'xp', 'y', 'yp', 'z', 'dp')}
        beam = Particles(n, 1., e, m_p, C_RING, GAMMA,
                         coords_n_momenta_dict=coords, precision=prec)
        del coords
        rec = torch.empty(34, dtype=torch.float64, device='cuda')
        for label, order, mask, nq in (('centroids x y', 1, 0x5, 2),
                                       ('centroids, six', 1, 0x3f, 6),
                                       ('order 2', 2, 0x3f, 6)):
            ms = []
            for it in range(a.warmup + a.steps):
                flush_l2(flush)
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record()
                beam.launch_stats(rec, order=order, mask=mask)
                e1.record()
                torch.cuda.synchronize()
                if it >= a.warmup:
                    ms.append(e0.elapsed_time(e1))
            t = float(np.median(ms))
            gbs = n * nq * beam.x.element_size() / (t * 1e-3) / 1e9
            cases['%s %s' % (prec, label)] = {
                'ms': t, 'particles_per_s': n / (t * 1e-3), 'GB/s': gbs,
                'frac_of_hbm': gbs / peak, 'peak_kind': peak_kind}
        del beam
        torch.cuda.empty_cache()
    head = cases.get('fp32 centroids, six') or next(iter(cases.values()))
    print(json.dumps({
        'metric': 'bunch statistics pass: particles/s', 'value':
        head['particles_per_s'], 'unit': 'particles/s', 'n_gpus': 1,
        'steps': a.steps, 'warmup': a.warmup,
        'config': {'n_macroparticles': n, 'l2': 'flushed between passes'},
        'cases': cases}))


# ------------------------------------------------------------ reference arm

def run_reference(a, rank, world):
    if rank != 0:
        return
    w = WORKLOADS[a.workload]
    coords = bunch_coords(w)
    ns = w['n']
    beam, els = build_oracle(w, coords)
    for _ in range(a.warmup):
        for m in els:
            m.track(beam)
    t0 = time.perf_counter()
    for _ in range(a.steps):
        for m in els:
            m.track(beam)
    dt = time.perf_counter() - t0
    v = ns * a.steps / dt
    sample = ('the full seeded bunch (%d macroparticles), one turn per step '
              '(oracle: NumPy restatement of the reference, single thread '
              'like the reference)' % ns)
    print(json.dumps({
        'impl': 'reference',
        'metric': 'macroparticle-turns/s on 1 GB300: FP32/batched vs FP64 '
                  'plain; % HBM roofline',
        'value': v, 'unit': 'macroparticle-turns/s', 'n_gpus': world,
        'steps': a.steps, 'warmup': a.warmup,
        'ms_per_step': dt / a.steps * 1e3, 'higher_is_better': True,
        'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f64',
        'data': 'synthetic: seeded 6D Gaussian bunch (reference generator '
                'draw order), no dataset',
        'config': bench_config(w), 'form': 'fp64', 'turns_per_step': 1,
        'cpu_baseline': {'value': v, 'unit': 'macroparticle-turns/s',
                         'cores': 1, 'kind': 'port', 'sample': sample,
                         'host': host_cpu()},
        'e2e': {'value': v, 'unit': 'macroparticle-turns/s',
                'h2d_bytes_per_step': 0, 'd2h_bytes_per_step': 0},
    }))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--gpus', type=int, default=1)
    ap.add_argument('--steps', type=int, default=400)
    ap.add_argument('--warmup', type=int, default=5)
    ap.add_argument('--impl', choices=['ours', 'reference'], default='ours')
    ap.add_argument('--workload', choices=sorted(WORKLOADS) + ['c4'],
                    default='c3')
    ap.add_argument('--form', choices=['all', 'fp64', 'fp32'], default='all')
    ap.add_argument('--no-cpu-baseline', action='store_true')
    ap.add_argument('--no-autotune', dest='autotune', action='store_false',
                    help='skip timing the launch shapes (FP32 pass, '
                         'batched workload)')
    ap.add_argument('--stats-pass', action='store_true',
                    help='time the bunch statistics pass instead of the turn')
    ap.add_argument('--shard', action='store_true',
                    help='split one bunch over the GPUs (particles; slice '
                         'sums merged every turn) instead of one replica '
                         'per GPU')
    ap.add_argument('--plan', default=None,
                    help='variant,stages,smem_kb: launch plan of the FP32 '
                         'pass (phk_set_track_plan) instead of the default '
                         'or the tuned one')
    ap.add_argument('--eager-turns', type=int, default=0,
                    help='run this many eager turns of the workload and '
                         'exit (a short run for profilers; no timing loop)')
    a = ap.parse_args()
    a.steps_given = any(x == '--steps' or x.startswith('--steps=')
                        for x in sys.argv[1:])
    a.warmup = max(3, a.warmup)
    world = int(os.environ.get('WORLD_SIZE', '1'))
    rank = int(os.environ.get('RANK', '0'))
    if a.stats_pass and a.impl == 'ours':
        return run_stats_pass(a, rank, world)
    if a.plan and a.impl == 'ours':
        from pyheadtail_gb300 import _native as N
        N.call('phk_set_track_plan', *[int(x) for x in a.plan.split(',')])
        a.autotune = False
    if a.eager_turns and a.impl == 'ours':
        return run_eager(a)
    if a.impl == 'reference':
        if a.workload == 'c4':
            return run_reference_c4(a, rank, world)
        return run_reference(a, rank, world)
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(int(os.environ.get('LOCAL_RANK', rank)))
        dist.init_process_group('nccl')
        dist.barrier()
    if a.workload == 'c4':
        run_batch(a, rank, world)
    elif a.shard:
        run_sharded(a, rank, world)
    else:
        run_ours(a, rank, world)
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
        dist.destroy_process_group()


if __name__ == '__main__':
    main()
