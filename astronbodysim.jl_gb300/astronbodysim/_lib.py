"""ctypes binding of libnbody_gb300.so (declarations in include/nbody_gb300.h).

The shared library is the only compute path: if it is missing or fails to load,
every call raises.  There is no CPU fallback.
"""
import ctypes
import os

import numpy as np

from . import _build

NB_OK = 0
NB_ERR_INVALID_ARG = -1
NB_ERR_OOM = -2
NB_ERR_CUDA = -3
NB_ERR_NUMERIC = -4
NB_ERR_TIMEOUT = -5
NB_ERR_ADMISSION = -6
NB_ERR_STATE = -7
NB_ERR_NOT_FOUND = -8

NB_LAW_SPLINE_G2 = 0
NB_LAW_PLUMMER = 1
NB_PREC_FP64 = 0
NB_PREC_MIXED = 1
NB_CRIT_REF = 0
NB_CRIT_ETA_SQRT_EPS = 1
NB_FORCE_POT = 1
NB_ALG_LEAPFROG = 0
NB_ALG_EULER = 1

_ERRNAMES = {
    NB_ERR_INVALID_ARG: "NB_ERR_INVALID_ARG", NB_ERR_OOM: "NB_ERR_OOM", NB_ERR_CUDA: "NB_ERR_CUDA",
    NB_ERR_NUMERIC: "NB_ERR_NUMERIC", NB_ERR_TIMEOUT: "NB_ERR_TIMEOUT",
    NB_ERR_ADMISSION: "NB_ERR_ADMISSION", NB_ERR_STATE: "NB_ERR_STATE",
    NB_ERR_NOT_FOUND: "NB_ERR_NOT_FOUND",
}


class NbodyError(RuntimeError):
    """Non-zero status from the C ABI; `code` is the NB_ERR_* value."""

    def __init__(self, code, msg):
        super().__init__("%s (%d): %s" % (_ERRNAMES.get(code, "NB_ERR"), code, msg))
        self.code = code


class nb_params(ctypes.Structure):
    _fields_ = [
        ("G", ctypes.c_double),
        ("softening", ctypes.c_double * 6),
        ("law", ctypes.c_int32),
        ("precision", ctypes.c_int32),
        ("adaptive", ctypes.c_int32),
        ("criterion", ctypes.c_int32),
        ("dt", ctypes.c_double),
        ("eta", ctypes.c_double),
        ("min_step", ctypes.c_double),
        ("max_step", ctypes.c_double),
        ("time_base", ctypes.c_int64),
        ("time_begin", ctypes.c_double),
        ("time_end", ctypes.c_double),
        ("device", ctypes.c_int32),
        ("tile_j", ctypes.c_int32),
        ("i_per_thread", ctypes.c_int32),
        ("block", ctypes.c_int32),
        ("j_split", ctypes.c_int32),
        ("algorithm", ctypes.c_int32),
        ("bg_kind", ctypes.c_int32),
        ("mond", ctypes.c_int32),
        ("bg_gm", ctypes.c_double),
        ("bg_center", ctypes.c_double * 3),
        ("bg_rg", ctypes.c_double),
        ("mond_acc0", ctypes.c_double),
        ("mond_nu_index", ctypes.c_double),
        ("stages", ctypes.c_int32),
        ("resort_every", ctypes.c_int32),
    ]


class nb_engine_params(ctypes.Structure):
    _fields_ = [
        ("G", ctypes.c_double),
        ("law", ctypes.c_int32),
        ("device", ctypes.c_int32),
        ("max_particles", ctypes.c_int64),
        ("max_systems", ctypes.c_int32),
        ("max_steps_per_call", ctypes.c_int32),
        ("block", ctypes.c_int32),
        ("i_per_thread", ctypes.c_int32),
    ]


class nb_engine_stats(ctypes.Structure):
    _fields_ = [
        ("queued", ctypes.c_int64),
        ("running", ctypes.c_int64),
        ("done", ctypes.c_int64),
        ("resident_particles", ctypes.c_int64),
        ("engine_steps", ctypes.c_int64),
        ("interactions", ctypes.c_double),
        ("gpu_ms", ctypes.c_double),
    ]


NB_REQ_QUEUED = 0
NB_REQ_RUNNING = 1
NB_REQ_DONE = 2
NB_REQ_CANCELLED = 3
NB_REQ_SUSPENDED = 4
NB_BG_NONE = 0
NB_BG_POINT_MASS = 1
NB_BG_PSEUDO_NEWTONIAN = 2
NB_MOND_NONE = 0
NB_MOND_MILGROM1983 = 1


class nb_diag(ctypes.Structure):
    _fields_ = [
        ("kinetic", ctypes.c_double),
        ("potential", ctypes.c_double),
        ("momentum", ctypes.c_double * 3),
        ("angular_momentum", ctypes.c_double * 3),
    ]


_dp = ctypes.POINTER(ctypes.c_double)
_i32p = ctypes.POINTER(ctypes.c_int32)
_i64p = ctypes.POINTER(ctypes.c_int64)
_vp = ctypes.c_void_p
_h = ctypes.c_void_p

# name -> (restype, argtypes); every name here is declared in include/nbody_gb300.h
SIGNATURES = {
    "nb_default_params": (None, [ctypes.POINTER(nb_params)]),
    "nb_create": (ctypes.c_int, [ctypes.POINTER(nb_params), ctypes.POINTER(_h)]),
    "nb_destroy": (ctypes.c_int, [_h]),
    "nb_set_stream": (ctypes.c_int, [_h, _vp]),
    "nb_get_stream": (ctypes.c_int, [_h, ctypes.POINTER(_vp)]),
    "nb_upload": (ctypes.c_int, [_h, ctypes.c_int64, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _i32p]),
    "nb_download": (ctypes.c_int, [_h, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _i64p, _i64p]),
    "nb_upload_acc": (ctypes.c_int, [_h, _dp, _dp, _dp]),
    "nb_upload_bins": (ctypes.c_int, [_h, _i64p, _i64p]),
    "nb_set_softening": (ctypes.c_int, [_h, _dp]),
    "nb_compute_force": (ctypes.c_int, [_h, ctypes.c_int]),
    "nb_compute_potential": (ctypes.c_int, [_h]),
    "nb_remove_self_potential": (ctypes.c_int, [_h]),
    "nb_force_at_points": (ctypes.c_int, [_h, ctypes.c_int64, _dp, _dp, _dp, ctypes.c_double, _dp, _dp, _dp, _dp]),
    "nb_init_timesteps": (ctypes.c_int, [_h]),
    "nb_half_kick": (ctypes.c_int, [_h, ctypes.c_int]),
    "nb_kick": (ctypes.c_int, [_h]),
    "nb_find_min_endstep": (ctypes.c_int, [_h, _i64p]),
    "nb_drift_to_int": (ctypes.c_int, [_h, ctypes.c_int64]),
    "nb_drift_to_float": (ctypes.c_int, [_h, ctypes.c_double]),
    "nb_step": (ctypes.c_int, [_h, ctypes.c_int64]),
    "nb_run_begin": (ctypes.c_int, [_h]),
    "nb_run_end": (ctypes.c_int, [_h]),
    "nb_set_snapshot_interval": (ctypes.c_int, [_h, ctypes.c_double]),
    "nb_step_until_output": (ctypes.c_int, [_h, ctypes.c_int64, _i64p, _i32p]),
    "nb_get_output_time": (ctypes.c_int, [_h, _i64p, _dp, _i32p, _i64p]),
    "nb_get_time": (ctypes.c_int, [_h, _i64p, _dp]),
    "nb_diagnostics": (ctypes.c_int, [_h, ctypes.c_int, ctypes.POINTER(nb_diag)]),
    "nb_active_count": (ctypes.c_int, [_h, _i64p]),
    "nb_get_counters": (ctypes.c_int, [_h, _i64p, _dp]),
    "nb_check_sync_point": (ctypes.c_int, [_h, ctypes.POINTER(ctypes.c_int32)]),
    "nb_batch_suspend": (ctypes.c_int, [_h, ctypes.c_int64]),
    "nb_batch_resume": (ctypes.c_int, [_h, ctypes.c_int64]),
    "nb_selftest_wait_timeout": (ctypes.c_int, [ctypes.c_int, ctypes.c_int64, _dp]),
    "nb_selftest_fp32_peak": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, _dp, _dp]),
    "nb_checkpoint_size": (ctypes.c_int, [_h, _i64p]),
    "nb_checkpoint_save": (ctypes.c_int, [_h, _vp, ctypes.c_int64]),
    "nb_checkpoint_load": (ctypes.c_int, [_h, _vp, ctypes.c_int64]),
    "nb_force_noalloc": (ctypes.c_int, [ctypes.c_int64, _vp, _vp, _vp, _vp, ctypes.c_int32,
                                        ctypes.c_double, ctypes.c_double, _vp, _vp, _vp, _vp, _vp,
                                        ctypes.c_char_p, ctypes.c_int64]),
    "nb_engine_create": (ctypes.c_int, [ctypes.POINTER(nb_engine_params), ctypes.POINTER(_h)]),
    "nb_engine_destroy": (ctypes.c_int, [_h]),
    "nb_batch_submit": (ctypes.c_int, [_h, ctypes.c_int64, _dp, _dp, _dp, _dp, _dp, _dp, _dp,
                                       ctypes.c_double, ctypes.c_double, ctypes.c_int64, _i64p]),
    "nb_engine_run": (ctypes.c_int, [_h, ctypes.c_int64, _i64p]),
    "nb_engine_run_async": (ctypes.c_int, [_h, ctypes.c_int64, _i64p]),
    "nb_engine_sync": (ctypes.c_int, [_h]),
    "nb_batch_poll": (ctypes.c_int, [_h, ctypes.c_int64, _i32p, _i64p]),
    "nb_batch_fetch": (ctypes.c_int, [_h, ctypes.c_int64, _dp, _dp, _dp, _dp, _dp, _dp]),
    "nb_batch_cancel": (ctypes.c_int, [_h, ctypes.c_int64]),
    "nb_engine_get_stats": (ctypes.c_int, [_h, ctypes.POINTER(nb_engine_stats)]),
    "nb_engine_drain_done": (ctypes.c_int, [_h, _i64p, ctypes.c_int64, _i64p]),
    "nb_engine_last_error": (ctypes.c_char_p, [_h]),
    "nb_last_error": (ctypes.c_char_p, [_h]),
    "nb_version": (ctypes.c_char_p, []),
}

_lib = None


def library_path():
    return _build.LIB


def load(build_if_missing=True):
    """Load libnbody_gb300.so (building it in place if asked and absent)."""
    global _lib
    if _lib is not None:
        return _lib
    path = library_path()
    if not os.path.exists(path):
        if not build_if_missing:
            raise ImportError("libnbody_gb300.so not built at %s" % path)
        _build.build_library()
    L = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def check(h, rc):
    if rc != NB_OK:
        msg = load().nb_last_error(h)
        raise NbodyError(rc, msg.decode() if msg else "")


def dptr(a):
    if a is None:
        return _dp()
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_dp)


def i64ptr(a):
    if a is None:
        return _i64p()
    assert a.dtype == np.int64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_i64p)


def i32ptr(a):
    if a is None:
        return _i32p()
    assert a.dtype == np.int32 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_i32p)
