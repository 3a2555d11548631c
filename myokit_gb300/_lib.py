"""
ctypes binding of the C ABI in ``include/mkg_tissue.h``.

The Python side of the simulation reaches the GPU only through these calls.
There is no CPU fallback: if the library is missing it is built, and if it
cannot be built or loaded an ``ImportError`` is raised.
"""
import ctypes
import os

import numpy as np

from . import build as _build

MKG_OK = 0
MKG_DONE = 1
MKG_HALT_NAN = 2
MKG_ERR_ARG = -1
MKG_ERR_CUDA = -2
MKG_ERR_COMPILE = -3
MKG_ERR_PACING = -4
MKG_ERR_TIMEOUT = -5
MKG_ERR_ORDER = -6
MKG_ERR_SIMULTANEOUS = -7
MKG_ERR_NOMEM = -8

PACE_ALL = 0
PACE_RECT = 1
PACE_LIST = 2
PACE_NONE = 3

_c_double_p = ctypes.POINTER(ctypes.c_double)
_c_int32_p = ctypes.POINTER(ctypes.c_int32)
_c_int64_p = ctypes.POINTER(ctypes.c_int64)


class MkgConfig(ctypes.Structure):
    """Mirror of ``mkg_config``."""
    _fields_ = [
        ('nx', ctypes.c_int64),
        ('ny', ctypes.c_int64),
        ('real_bytes', ctypes.c_int32),
        ('n_state', ctypes.c_int32),
        ('n_inter', ctypes.c_int32),
        ('n_field', ctypes.c_int32),
        ('i_vm', ctypes.c_int32),
        ('diffusion', ctypes.c_int32),
        ('block_x', ctypes.c_int32),
        ('block_y', ctypes.c_int32),
        ('device', ctypes.c_int32),
        ('two_d', ctypes.c_int32),
        ('hi_mode', ctypes.c_int32),
        ('n_hi', ctypes.c_int32),
        ('stage', ctypes.c_int32),
        ('v_double', ctypes.c_int32),
        ('split', ctypes.c_int32),
    ]


# Every symbol declared in include/mkg_tissue.h, with its signature
SIGNATURES = {
    'mkg_set_wait': (ctypes.c_int, [
        ctypes.c_void_p, ctypes.c_int64, ctypes.c_int32]),
    'mkg_set_partner': (ctypes.c_int, [
        ctypes.c_void_p, ctypes.c_void_p, ctypes.c_double, ctypes.c_int64]),
    'mkg_stage_layout': (ctypes.c_int, [
        ctypes.POINTER(MkgConfig), ctypes.POINTER(ctypes.c_int64)]),
    'mkg_compile': (ctypes.c_int, [
        ctypes.c_char_p, ctypes.c_char_p, ctypes.POINTER(ctypes.c_char_p),
        ctypes.c_int, ctypes.POINTER(ctypes.c_void_p),
        ctypes.POINTER(ctypes.c_size_t), ctypes.POINTER(ctypes.c_void_p)]),
    'mkg_free': (None, [ctypes.c_void_p]),
    'mkg_create': (ctypes.c_int, [
        ctypes.POINTER(MkgConfig), ctypes.c_void_p, ctypes.c_size_t,
        ctypes.POINTER(ctypes.c_void_p)]),
    'mkg_destroy': (None, [ctypes.c_void_p]),
    'mkg_last_error': (ctypes.c_char_p, [ctypes.c_void_p]),
    'mkg_set_state': (ctypes.c_int, [
        ctypes.c_void_p, _c_double_p, ctypes.c_int64]),
    'mkg_set_hi_states': (ctypes.c_int, [
        ctypes.c_void_p, _c_int32_p, ctypes.c_int32]),
    'mkg_set_state_static': (ctypes.c_int, [
        ctypes.c_void_p, _c_double_p, ctypes.c_int64]),
    'mkg_get_state': (ctypes.c_int, [
        ctypes.c_void_p, _c_double_p, ctypes.c_int64]),
    'mkg_set_fields': (ctypes.c_int, [
        ctypes.c_void_p, _c_double_p, ctypes.c_int64]),
    'mkg_set_conductance': (ctypes.c_int, [
        ctypes.c_void_p, ctypes.c_double, ctypes.c_double]),
    'mkg_set_conductance_field': (ctypes.c_int, [
        ctypes.c_void_p, _c_double_p, ctypes.c_int64, _c_double_p,
        ctypes.c_int64]),
    'mkg_set_connections': (ctypes.c_int, [
        ctypes.c_void_p, _c_int64_p, _c_int64_p, _c_double_p,
        ctypes.c_int64]),
    'mkg_set_pacing_mode': (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32]),
    'mkg_set_paced_rect': (ctypes.c_int, [
        ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64,
        ctypes.c_int64]),
    'mkg_set_paced_list': (ctypes.c_int, [
        ctypes.c_void_p, _c_int64_p, ctypes.c_int64]),
    'mkg_set_protocol': (ctypes.c_int, [
        ctypes.c_void_p, _c_double_p, ctypes.c_int64]),
    'mkg_set_log': (ctypes.c_int, [
        ctypes.c_void_p, _c_int32_p, _c_int64_p, ctypes.c_int64,
        ctypes.c_int32]),
    'mkg_run_begin': (ctypes.c_int, [
        ctypes.c_void_p, ctypes.c_double, ctypes.c_double, ctypes.c_double,
        ctypes.c_double]),
    'mkg_run_chunk': (ctypes.c_int, [
        ctypes.c_void_p, ctypes.c_int64, _c_double_p, _c_int64_p]),
    'mkg_read_log': (ctypes.c_int, [
        ctypes.c_void_p, _c_double_p, _c_double_p, _c_double_p,
        ctypes.c_int64]),
    'mkg_set_tuning': (ctypes.c_int, [
        ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32]),
    'mkg_last_stats': (ctypes.c_int, [
        ctypes.c_void_p, _c_double_p, _c_int64_p, _c_int64_p]),
    'mkg_launch_count': (ctypes.c_int, [ctypes.c_void_p, _c_int64_p]),
    'mkg_set_frame_buffer': (ctypes.c_int, [
        ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64]),
    'mkg_adj_attach': (ctypes.c_int, [
        ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int32]),
    'mkg_adj_forward': (ctypes.c_int, [
        ctypes.c_void_p, ctypes.c_double, ctypes.c_double, ctypes.c_double,
        ctypes.c_double, _c_int64_p]),
    'mkg_adj_read_log': (ctypes.c_int, [
        ctypes.c_void_p, _c_double_p, ctypes.c_int64]),
    'mkg_adj_backward': (ctypes.c_int, [
        ctypes.c_void_p, _c_double_p, ctypes.c_int64, _c_double_p,
        _c_double_p]),
    'mkg_adj_conductance_gradient': (ctypes.c_int, [
        ctypes.c_void_p, _c_double_p, ctypes.c_int64]),
    'mkg_stream': (ctypes.c_int, [
        ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p)]),
    'mkg_schedule_preview': (ctypes.c_int64, [
        _c_double_p, ctypes.c_int64, ctypes.c_double, ctypes.c_double,
        ctypes.c_double, ctypes.c_double, ctypes.c_int64, _c_double_p,
        _c_double_p, _c_double_p, _c_int32_p]),
}

_lib = None


def load():
    """Loads (building first if needed) and returns the host library."""
    global _lib
    if _lib is not None:
        return _lib
    try:
        path = _build.build()
    except Exception as e:
        if not os.path.exists(_build.LIB_PATH):
            raise ImportError('Cannot build libmkg_tissue.so: ' + str(e))
        path = _build.LIB_PATH
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def dptr(a):
    """Pointer to a C-contiguous float64 numpy array (or None)."""
    if a is None:
        return None
    return a.ctypes.data_as(_c_double_p)


def i64ptr(a):
    return None if a is None else a.ctypes.data_as(_c_int64_p)


def i32ptr(a):
    return None if a is None else a.ctypes.data_as(_c_int32_p)


class MkgError(RuntimeError):
    """An error status returned by the host library."""
    def __init__(self, code, message):
        super().__init__(message)
        self.code = code


def check(code, handle=None):
    """Raises MkgError for a negative status; returns the status."""
    if code < 0:
        msg = load().mkg_last_error(handle)
        msg = msg.decode('utf-8', 'replace') if msg else 'unknown error'
        raise MkgError(code, msg)
    return code


def compile_source(source, options, name='mkg_tissue.cu'):
    """Compiles CUDA source to a cubin (bytes) with NVRTC."""
    lib = load()
    opts = (ctypes.c_char_p * len(options))(*[o.encode() for o in options])
    cubin = ctypes.c_void_p()
    size = ctypes.c_size_t()
    log = ctypes.c_void_p()
    code = lib.mkg_compile(
        source.encode(), name.encode(), opts, len(options),
        ctypes.byref(cubin), ctypes.byref(size), ctypes.byref(log))
    text = ''
    if log.value:
        text = ctypes.cast(log, ctypes.c_char_p).value.decode(
            'utf-8', 'replace')
        lib.mkg_free(log)
    if code < 0:
        msg = lib.mkg_last_error(None).decode('utf-8', 'replace')
        raise MkgError(code, msg)
    data = ctypes.string_at(cubin, size.value)
    lib.mkg_free(cubin)
    return data, text


def schedule_preview(events, tmin, tmax, dt, log_interval, max_steps):
    """Returns the (t, dt, pace, log) arrays of the host step schedule."""
    lib = load()
    ev = np.ascontiguousarray(events, dtype=np.float64).reshape(-1, 5)
    t = np.zeros(max_steps)
    d = np.zeros(max_steps)
    p = np.zeros(max_steps)
    lg = np.zeros(max_steps, dtype=np.int32)
    n = lib.mkg_schedule_preview(
        dptr(ev), len(ev), tmin, tmax, dt, log_interval, max_steps,
        dptr(t), dptr(d), dptr(p), i32ptr(lg))
    if n < 0:
        raise MkgError(int(n), 'pacing error %d' % n)
    return t[:n], d[:n], p[:n], lg[:n].astype(bool)
