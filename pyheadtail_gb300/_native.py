"""ctypes binding of libphk.so (include/pyheadtail_gb300.h).

The structures below mirror the C parameter blocks field for field.  Every
call checks the returned status and raises ``PhkError`` with the library's
message; there is no fallback -- when the library or a CUDA device is
missing, using the GPU path raises.
"""
import ctypes
import os

from . import _build

PHK_F64, PHK_F32 = 0, 1
PHK_DEV_TIMEOUT = 1
PHK_DEV_TIMEOUT_UNDRAINED = 4
PHK_DEV_BAD_TABLE = 2
PHK_MAX_OPS = 12
PHK_MAX_DETUNERS = 6
PHK_MAX_POLY = 8
PHK_MAX_KICKS = 8
PHK_MAX_SLICES = 4096
PHK_X, PHK_XP, PHK_Y, PHK_YP, PHK_Z, PHK_DP = range(6)
COORD_INDEX = {'x': PHK_X, 'xp': PHK_XP, 'y': PHK_Y, 'yp': PHK_YP,
               'z': PHK_Z, 'dp': PHK_DP}

OP_TRANSVERSE, OP_DRIFT, OP_RF_KICK, OP_LINEAR_LONG, OP_SCALE_TRANS = 1, 2, 3, 4, 5
OP_DAMPER = 6
FLAG_DISPERSION, FLAG_DETUNED, FLAG_SHRINK = 1, 2, 4
FLAG_PHI_OFFSET, FLAG_PHI_LOCK, FLAG_P_INC = 8, 16, 32
FLAG_DAMP_X, FLAG_DAMP_Y, FLAG_REACTIVE = 64, 128, 256
DET_CHROMA, DET_AMPLITUDE = 1, 2

c_double_p = ctypes.POINTER(ctypes.c_double)
c_int32_p = ctypes.POINTER(ctypes.c_int32)


class Coords(ctypes.Structure):
    _fields_ = [('x', ctypes.c_void_p), ('xp', ctypes.c_void_p),
                ('y', ctypes.c_void_p), ('yp', ctypes.c_void_p),
                ('z', ctypes.c_void_p), ('dp', ctypes.c_void_p),
                ('n', ctypes.c_int64), ('dtype', ctypes.c_int32),
                ('reserved', ctypes.c_int32)]


class Slicer(ctypes.Structure):
    _fields_ = [('n_slices', ctypes.c_int32), ('negate', ctypes.c_int32),
                ('tail', ctypes.c_double), ('width', ctypes.c_double),
                ('est_tail', ctypes.c_double), ('est_inv_w', ctypes.c_double),
                ('edges', ctypes.c_void_p)]


class Op(ctypes.Structure):
    _fields_ = [('kind', ctypes.c_int32), ('flags', ctypes.c_int32),
                ('det_begin', ctypes.c_int32), ('det_count', ctypes.c_int32),
                ('ij_mask', ctypes.c_int32), ('reserved', ctypes.c_int32),
                ('p', ctypes.c_double * 32)]


class Detuner(ctypes.Structure):
    _fields_ = [('kind', ctypes.c_int32), ('nx', ctypes.c_int32),
                ('ny', ctypes.c_int32), ('zx', ctypes.c_int32),
                ('zy', ctypes.c_int32), ('reserved', ctypes.c_int32),
                ('c', ctypes.c_double * 16)]


class Program(ctypes.Structure):
    _fields_ = [('n_ops', ctypes.c_int32), ('n_det', ctypes.c_int32),
                ('op', Op * PHK_MAX_OPS), ('det', Detuner * PHK_MAX_DETUNERS),
                ('status', ctypes.c_void_p)]


class KickSet(ctypes.Structure):
    _fields_ = [('slicer', Slicer), ('n_kicks', ctypes.c_int32),
                ('target', ctypes.c_int32 * PHK_MAX_KICKS),
                ('quad', ctypes.c_int32 * PHK_MAX_KICKS),
                ('kick', ctypes.c_void_p * PHK_MAX_KICKS)]


class Accum(ctypes.Structure):
    _fields_ = [('slicer', Slicer), ('partials', ctypes.c_void_p),
                ('partials_len', ctypes.c_int64), ('idx_out', ctypes.c_void_p),
                ('grid', ctypes.c_int32), ('reserved', ctypes.c_int32)]


class WakeKick(ctypes.Structure):
    _fields_ = [('source', ctypes.c_int32), ('n_lags', ctypes.c_int32),
                ('dense', ctypes.c_int32), ('reserved', ctypes.c_int32),
                ('factor', ctypes.c_double), ('table', ctypes.c_void_p),
                ('out', ctypes.c_void_p)]


class WakeSet(ctypes.Structure):
    _fields_ = [('n_slices', ctypes.c_int32), ('ring_len', ctypes.c_int32),
                ('head', ctypes.c_int32), ('n_kicks', ctypes.c_int32),
                ('out_dtype', ctypes.c_int32), ('reserved', ctypes.c_int32),
                ('moments', ctypes.c_void_p),
                ('kick', WakeKick * PHK_MAX_KICKS)]


class WakeTC(ctypes.Structure):
    _fields_ = [('n_slices', ctypes.c_int32), ('ring_len', ctypes.c_int32),
                ('head', ctypes.c_int32), ('n_kicks', ctypes.c_int32),
                ('n_groups', ctypes.c_int32), ('k_total', ctypes.c_int32),
                ('m_tiles', ctypes.c_int32), ('splits', ctypes.c_int32),
                ('out_dtype', ctypes.c_int32), ('reserved', ctypes.c_int32),
                ('group_lags', ctypes.c_int32 * PHK_MAX_KICKS),
                ('group_k0', ctypes.c_int32 * PHK_MAX_KICKS),
                ('group_of', ctypes.c_int32 * PHK_MAX_KICKS),
                ('source', ctypes.c_int32 * PHK_MAX_KICKS),
                ('n_lags', ctypes.c_int32 * PHK_MAX_KICKS),
                ('factor', ctypes.c_double * PHK_MAX_KICKS),
                ('tables', ctypes.c_void_p * PHK_MAX_KICKS),
                ('out', ctypes.c_void_p * PHK_MAX_KICKS),
                ('moments', ctypes.c_void_p), ('a_hi', ctypes.c_void_p),
                ('a_lo', ctypes.c_void_p), ('partials', ctypes.c_void_p),
                ('status', ctypes.c_void_p)]


class Unit(ctypes.Structure):
    _fields_ = [('start', ctypes.c_int64), ('end', ctypes.c_int64),
                ('bunch', ctypes.c_int32), ('column', ctypes.c_int32)]


class Batch(ctypes.Structure):
    _fields_ = [('n_bunches', ctypes.c_int32), ('n_units', ctypes.c_int32),
                ('n_columns', ctypes.c_int32), ('grid', ctypes.c_int32),
                ('threads', ctypes.c_int32), ('reserved', ctypes.c_int32),
                ('units', ctypes.c_void_p), ('cta_first', ctypes.c_void_p),
                ('programs', ctypes.c_void_p),
                ('programs_host', ctypes.POINTER(Program)),
                ('kicks', ctypes.c_void_p), ('status', ctypes.c_void_p)]


PHK_STATS_LEN = 34


class Stats(ctypes.Structure):
    _fields_ = [('order', ctypes.c_int32), ('capacity', ctypes.c_int32),
                ('records', ctypes.c_void_p), ('cursor', ctypes.c_void_p),
                ('partials', ctypes.c_void_p), ('ticket', ctypes.c_void_p),
                ('means', ctypes.c_void_p),
                ('grid', ctypes.c_int32), ('mask', ctypes.c_int32)]


class PhkError(RuntimeError):
    """A libphk entry point returned a non-zero status."""


# name -> (argtypes); every entry point returns int
SIGNATURES = {
    'phk_abi_version': [],
    'phk_set_wait_limit': [ctypes.c_int64],
    'phk_launch_count': [],
    'phk_last_error': [ctypes.c_char_p, ctypes.c_int],
    'phk_track_grid': [ctypes.c_int64, ctypes.c_int32, ctypes.c_int32],
    'phk_track': [ctypes.POINTER(Program), ctypes.POINTER(Coords),
                  ctypes.POINTER(KickSet), ctypes.POINTER(Accum),
                  ctypes.c_void_p],
    'phk_slice_finalize': [ctypes.POINTER(Accum), ctypes.c_void_p,
                           ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                           ctypes.c_void_p],
    'phk_wake': [ctypes.POINTER(WakeSet), ctypes.c_void_p],
    'phk_kick': [ctypes.POINTER(Coords), ctypes.POINTER(KickSet),
                 ctypes.c_void_p],
    'phk_slice_moments': [ctypes.POINTER(Slicer), ctypes.c_void_p,
                          ctypes.c_int64, ctypes.c_int32,
                          ctypes.POINTER(ctypes.c_void_p), ctypes.c_int32,
                          ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p,
                          ctypes.c_void_p, ctypes.c_void_p],
    'phk_track_batch': [ctypes.POINTER(Batch), ctypes.POINTER(Coords),
                        ctypes.POINTER(KickSet), ctypes.POINTER(Accum),
                        ctypes.c_void_p],
    'phk_batch_max_grid': [ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                           ctypes.c_int32],
    'phk_batch_finalize': [ctypes.POINTER(Accum), ctypes.c_int32,
                           ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                           ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64,
                           ctypes.c_void_p],
    'phk_wake_batch': [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32,
                       ctypes.c_int32, ctypes.c_void_p],
    'phk_wake_tc_plan': [ctypes.POINTER(WakeTC),
                         ctypes.POINTER(ctypes.c_int64),
                         ctypes.POINTER(ctypes.c_int64)],
    'phk_wake_tc_expand': [ctypes.POINTER(WakeTC), ctypes.c_void_p],
    'phk_set_track_plan': [ctypes.c_int32, ctypes.c_int32, ctypes.c_int32],
    'phk_slice_sums': [ctypes.POINTER(Accum), ctypes.c_void_p, ctypes.c_void_p],
    'phk_slice_merge': [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32,
                        ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                        ctypes.c_void_p, ctypes.c_void_p],
    'phk_last_track_launch': [ctypes.POINTER(ctypes.c_int32)] * 3,
    'phk_wake_tc_run': [ctypes.POINTER(WakeTC), ctypes.c_void_p],
    'phk_slice_noalloc': [ctypes.POINTER(Slicer), ctypes.POINTER(Coords),
                          ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                          ctypes.c_void_p],
    'phk_bunch_stats_grid': [ctypes.c_int64, ctypes.c_int32],
    'phk_charge_hist': [ctypes.c_void_p, ctypes.c_int64, ctypes.c_int32,
                        ctypes.c_double, ctypes.c_double, ctypes.c_int32,
                        ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p],
    'phk_charge_gather': [ctypes.c_void_p, ctypes.c_int64, ctypes.c_int32,
                          ctypes.c_double, ctypes.c_double, ctypes.c_int32,
                          ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                          ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                          ctypes.c_void_p],
    'phk_charge_select': [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                          ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32,
                          ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p],
    'phk_bunch_stats': [ctypes.POINTER(Coords), ctypes.POINTER(KickSet),
                        ctypes.POINTER(Stats), ctypes.c_void_p],
}

_lib = None


def library_path():
    return _build.LIB


def load(build_if_missing=True):
    """Load libphk.so (building it first when it is missing or stale and
    ``build_if_missing``); raise if that is impossible."""
    global _lib
    if _lib is not None:
        return _lib
    path = library_path()
    if build_if_missing:
        path = _build.build()
    if not os.path.exists(path):
        raise PhkError('libphk.so is not built (%s); run '
                       'python -m pyheadtail_gb300._build' % path)
    lib = ctypes.CDLL(path)
    for name, argtypes in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.argtypes = argtypes
        fn.restype = ctypes.c_int64 if name == 'phk_launch_count' \
            else ctypes.c_int
    if lib.phk_abi_version() != 1:
        raise PhkError('libphk ABI version mismatch')
    _lib = lib
    return lib


def launch_count():
    """Kernels launched by libphk in this process so far."""
    return int(load().phk_launch_count())


def last_error():
    buf = ctypes.create_string_buffer(512)
    load().phk_last_error(buf, 512)
    return buf.value.decode(errors='replace')


def check(status, what):
    if status < 0:
        raise PhkError('%s failed (status %d): %s' % (what, status,
                                                       last_error()))
    return status


# observers of native calls (pyheadtail_gb300.turngraph records the
# parameters of a turn to verify that it is stationary)
RECORDERS = []


def call(name, *args):
    for r in RECORDERS:
        r(name, args)
    return check(getattr(load(), name)(*args), name)
