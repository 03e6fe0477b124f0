"""Deferred execution of a beam's element sequence on the GPU.

``Element.track(beam)`` of the fusion-aware elements does not launch a
kernel: it evaluates the element's host scalars with the reference's
formulas (so ``beam.gamma``, ``beam.p0`` ... are exact after every call,
as in PyHEADTAIL) and appends an *op* to the beam's pending program.  The
program is executed in one pass over the particles by ``phk_track`` when a
result is needed:

* a coordinate is read or replaced (``beam.x`` ...),
* a slice set is requested (``get_slices`` / ``WakeField.track``): the
  pass then also bins the updated z and accumulates the per-slice sums,
* the program is full.

A WakeField leaves its kicks *pending*; the next pass applies them before
the program, so a turn ``[transverse, longitudinal, wake]`` costs one pass
over the coordinates plus a small wake kernel.  Only reads of xp / yp / dp
force a pending kick out on its own (``phk_kick``): x, y and z do not
depend on it.
"""
import ctypes

import numpy as np
import torch

from . import _native as N
from . import tuning

_F64, _F32 = N.PHK_F64, N.PHK_F32


def torch_dtype(code):
    return torch.float64 if code == _F64 else torch.float32


def np_dtype(code):
    return np.float64 if code == _F64 else np.float32


def stream_handle():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def require_cuda(t, what='tensor'):
    if not t.is_cuda:
        raise N.PhkError('%s must live on a CUDA device' % what)


# ---------------------------------------------------------------- slicing

def reference_index(z, tail, width):
    """int32(floor((z - tail)/width)) as UniformBinSlicer computes it
    (particles/slicing.py:609-611), evaluated in float64."""
    return np.floor((np.asarray(z, dtype=np.float64) - tail) / width)


def _ordered_keys(x):
    """Map floats to integers with the same order (sign-magnitude to two's
    complement); +0 and -0 both map to 0."""
    it = np.int64 if x.dtype == np.float64 else np.int32
    b = x.view(it).astype(np.int64)
    mag = b & (np.int64(2**63 - 1) if it is np.int64 else np.int64(2**31 - 1))
    return np.where(b < 0, -mag, b)


def _from_keys(k, dt):
    it = np.int64 if dt == np.float64 else np.int32
    sign = np.int64(-2**63) if it is np.int64 else np.int64(-2**31)
    b = np.where(k < 0, (-k) | sign, k).astype(it)
    return b.view(dt)


def exact_edges(tail, width, n_slices, code):
    """Lower slice boundaries e_k, k = 0..S, in the coordinate dtype:
    e_k is the smallest representable z with reference_index(z) >= k.

    The index is non-decreasing in z (rounded subtraction and division are
    monotone), so {z : index(z) >= k} = [e_k, inf) and the device index of
    a particle is the k with e_k <= z < e_{k+1}.  For width < 0 the index is
    non-decreasing in -z; the table is then built for u = -z (negation is
    exact, and (z - tail)/width == (-z - -tail)/(-width) bit for bit).
    Each e_k is found by bisection over the ordered float lattice."""
    dt = np_dtype(code)
    neg = width < 0
    ks = np.arange(n_slices + 1, dtype=np.float64)

    def ok(u):  # index(z(u)) >= k
        z = -u.astype(np.float64) if neg else u.astype(np.float64)
        with np.errstate(invalid='ignore', over='ignore'):
            return reference_index(z, tail, width) >= ks

    aw = abs(width)
    mid = (-(tail + ks * width)) if neg else (tail + ks * width)
    lo = (mid - aw).astype(dt)
    hi = (mid + aw).astype(dt)
    for _ in range(64):
        bad = ok(lo)
        if not bad.any():
            break
        lo[bad] = (lo[bad].astype(np.float64) - 4 * aw).astype(dt)
    for _ in range(64):
        bad = ~ok(hi)
        if not bad.any():
            break
        hi[bad] = (hi[bad].astype(np.float64) + 4 * aw).astype(dt)
    if ok(lo).any() or (~ok(hi)).any():
        raise N.PhkError('slice edge bracket failed (tail %r width %r)'
                         % (tail, width))
    klo, khi = _ordered_keys(lo), _ordered_keys(hi)
    while True:
        open_ = khi - klo > 1
        if not open_.any():
            break
        km = klo + (khi - klo) // 2
        good = ok(_from_keys(km, dt))
        khi = np.where(open_ & good, km, khi)
        klo = np.where(open_ & ~good, km, klo)
    return _from_keys(khi, dt), neg


def ceil_to_dtype(v, code):
    """The smallest value of the coordinate dtype that is >= v."""
    if code == _F64:
        return np.float64(v)
    f = np.float32(v)
    if np.float64(f) < v:
        f = np.nextafter(f, np.float32(np.inf))
    return f


class DeviceSlicer(object):
    """Exact bin tables of one (cuts, n_slices, dtype) on the device."""

    def __init__(self, tail, head, n_slices, code, device, edges=None):
        tail = float(tail)
        width = (head - tail) / float(n_slices)
        if edges is None:
            e, neg = exact_edges(tail, width, n_slices, code)
        else:
            # given lower edges (non-uniform slices), ascending in z
            e, neg = np.ascontiguousarray(edges, dtype=np_dtype(code)), False
        self.tail, self.head, self.width = tail, head, width
        self.n_slices = n_slices
        self.code = code
        self.edges = torch.from_numpy(e).to(device)
        self.struct = N.Slicer()
        self.struct.n_slices = n_slices
        self.struct.negate = int(neg)
        self.struct.tail = tail
        self.struct.width = width
        self.struct.est_tail = -tail if neg else tail
        self.struct.est_inv_w = 1.0 / abs(width) if width != 0 else 0.0
        self.struct.edges = self.edges.data_ptr()


# ---------------------------------------------------------------- ops

def split_ff(v):
    """float-float split of a float64: hi + lo == v to ~2^-48 relative."""
    hi = np.float32(v)
    lo = np.float32(v - np.float64(hi))
    return hi, lo


class Op(object):
    """One element step of a pending program.  ``p`` holds the FP64
    parameters in the layout of include/pyheadtail_gb300.h; ``pf`` (FP32
    form) the float parameters packed into the same 256 bytes."""

    def __init__(self, kind, flags=0, p=None, pf=None, detuners=(),
                 ij_mask=0, pointer=None):
        self.kind, self.flags = kind, flags
        self.p = p or {}
        self.pf = pf or {}
        self.detuners = list(detuners)   # list of (DetunerPack)
        self.ij_mask = ij_mask
        self.pointer = pointer           # device address stored in p[31]

    def pack(self, st, code, det_begin):
        st.kind = self.kind
        st.flags = self.flags
        st.det_begin = det_begin
        st.det_count = len(self.detuners)
        st.ij_mask = self.ij_mask
        if code == _F64:
            for k, v in self.p.items():
                st.p[k] = v
        else:
            buf = np.zeros(64, dtype=np.float32)
            for k, v in self.pf.items():
                buf[k] = v
            ctypes.memmove(ctypes.addressof(st.p), buf.ctypes.data, 256)
        if self.pointer is not None:
            ptr = ctypes.c_uint64(self.pointer)
            ctypes.memmove(ctypes.addressof(st.p) + 248, ctypes.addressof(ptr),
                           8)


class DetunerPack(object):
    """Detuner parameters for phk_detuner (FP64 ``c`` or FP32 ``cf``)."""

    def __init__(self, kind, c, cf, nx=0, ny=0, zx=0, zy=0):
        self.kind, self.c, self.cf = kind, c, cf
        self.nx, self.ny, self.zx, self.zy = nx, ny, zx, zy

    def pack(self, st, code):
        st.kind = self.kind
        st.nx, st.ny, st.zx, st.zy = self.nx, self.ny, self.zx, self.zy
        if code == _F64:
            for k, v in self.c.items():
                st.c[k] = v
        else:
            buf = np.zeros(32, dtype=np.float32)
            for k, v in self.cf.items():
                buf[k] = v
            ctypes.memmove(ctypes.addressof(st.c), buf.ctypes.data, 128)


class PendingKick(object):
    """Wake kicks waiting to be applied: slicer + (target, quad, tensor)."""

    def __init__(self, dslicer, kicks):
        self.dslicer = dslicer
        self.kicks = list(kicks)
        self.targets = {t for t, _, _ in self.kicks}

    def struct(self):
        ks = N.KickSet()
        ks.slicer = self.dslicer.struct
        ks.n_kicks = len(self.kicks)
        for i, (t, q, tensor) in enumerate(self.kicks):
            ks.target[i] = t
            ks.quad[i] = -1 if q is None else q
            ks.kick[i] = tensor.data_ptr()
        return ks

    def merged(self, other):
        if other.dslicer is not self.dslicer:
            return None
        if len(self.kicks) + len(other.kicks) > N.PHK_MAX_KICKS:
            return None
        return PendingKick(self.dslicer, self.kicks + other.kicks)


class AccumRequest(object):
    """Slice accumulation for a pass: slicer, partials workspace, index."""

    def __init__(self, dslicer, partials, grid, idx_out=None):
        self.dslicer, self.partials, self.grid = dslicer, partials, grid
        self.idx_out = idx_out

    def struct(self):
        a = N.Accum()
        a.slicer = self.dslicer.struct
        a.partials = self.partials.data_ptr()
        a.partials_len = self.partials.numel()
        a.idx_out = 0 if self.idx_out is None else self.idx_out.data_ptr()
        a.grid = self.grid
        return a


class Engine(object):
    """Pending program + pending kick of one beam."""

    def __init__(self, beam):
        self.beam = beam
        self.ops = []
        self.kick = None
        self._workspaces = {}
        self.launches = 0
        self.z_version = 0     # bumped whenever z may have changed
        # bumped whenever the beam's state (coordinates with the pending
        # program and kick applied) may have changed
        self.version = 0
        # optional list; when set, (start, end) CUDA events are recorded
        # around every fused track launch (used to time the kernel alone)
        self.track_events = None

    # -- building
    def touch(self):
        """Record that the coordinates were changed from outside."""
        self.version += 1

    def enqueue(self, op):
        self.version += 1
        self.ops.append(op)
        n_det = sum(len(o.detuners) for o in self.ops)
        if len(self.ops) >= N.PHK_MAX_OPS or n_det > N.PHK_MAX_DETUNERS - 2:
            self.flush()

    def set_kick(self, kick):
        self.version += 1
        if self.ops:
            self.flush()
        if self.kick is not None:
            m = self.kick.merged(kick)
            if m is not None:
                self.kick = m
                return
            self.flush()
        self.kick = kick

    # -- execution
    def coords_struct(self):
        b = self.beam
        c = N.Coords()
        t = b._c
        c.x, c.xp, c.y = t['x'].data_ptr(), t['xp'].data_ptr(), t['y'].data_ptr()
        c.yp, c.z, c.dp = t['yp'].data_ptr(), t['z'].data_ptr(), t['dp'].data_ptr()
        c.n = b.macroparticlenumber
        c.dtype = b._code
        return c

    def program_struct(self, ops):
        prog = N.Program()
        prog.n_ops = len(ops)
        det = 0
        for i, op in enumerate(ops):
            op.pack(prog.op[i], self.beam._code, det)
            for d in op.detuners:
                d.pack(prog.det[det], self.beam._code)
                det += 1
        prog.n_det = det
        return prog

    def workspace(self, n_slices):
        """Partials buffer and grid for accumulations over n_slices."""
        key = n_slices
        if key not in self._workspaces:
            b = self.beam
            grid = N.call('phk_track_grid', b.macroparticlenumber, b._code,
                          n_slices)
            part = torch.empty(3 * n_slices * grid, dtype=torch.float64,
                               device=b._device)
            self._workspaces[key] = (part, grid)
        return self._workspaces[key]

    def flush(self, acc=None):
        """Run the pending program (+ pending kick, + accumulation)."""
        if not self.ops and self.kick is None and acc is None:
            return
        prog = self.program_struct(self.ops)
        coords = self.coords_struct()
        ks = self.kick.struct() if self.kick is not None else None
        ac = acc.struct() if acc is not None else None
        ev = None
        if self.track_events is not None:
            ev = (torch.cuda.Event(enable_timing=True),
                  torch.cuda.Event(enable_timing=True))
            ev[0].record()
        self._set_plan(prog, coords, ks, ac, self.ops, self.kick, acc)
        N.call('phk_track', ctypes.byref(prog), ctypes.byref(coords),
               ctypes.byref(ks) if ks is not None else None,
               ctypes.byref(ac) if ac is not None else None, stream_handle())
        if ev is not None:
            ev[1].record()
            self.track_events.append(ev)
        self.launches += 1
        if self.ops:
            self.z_version += 1
        self.ops = []
        self.kick = None

    def _set_plan(self, prog, coords, ks, ac, ops, kick, acc):
        """With tuning on (pyheadtail_gb300.tuning), set the tuned launch
        plan of this FP32 pass; otherwise leave the process's plan as it
        is (the default unless phk_set_track_plan changed it)."""
        if self.beam._code != _F32 or not tuning.enabled():
            return
        plan = tuning.plan_for(self, prog, coords, ks, ac, ops, kick, acc,
                               stream_handle())
        N.call('phk_set_track_plan', *plan)

    def slice_pass(self, acc):
        """Slicing pass over the coordinates as they are in memory, leaving
        any pending program and kick pending (z is not affected by kicks)."""
        prog = self.program_struct([])
        coords = self.coords_struct()
        ac = acc.struct()
        self._set_plan(prog, coords, None, ac, [], None, acc)
        N.call('phk_track', ctypes.byref(prog), ctypes.byref(coords), None,
               ctypes.byref(ac), stream_handle())
        self.launches += 1

    def flush_kick_only(self):
        ks = self.kick.struct()
        coords = self.coords_struct()
        N.call('phk_kick', ctypes.byref(coords), ctypes.byref(ks),
               stream_handle())
        self.launches += 1
        self.kick = None

    def sync_for(self, name):
        """Make coordinate ``name`` current before it is exposed."""
        if self.ops:
            self.flush()
        elif self.kick is not None and N.COORD_INDEX[name] in self.kick.targets:
            self.flush_kick_only()

    @property
    def idle(self):
        return not self.ops and self.kick is None
