"""ctypes binding of libcs_gb300.so (the C ABI in include/cs_gb300.h).

The library is built in tree by build.py.  There is no CPU fallback: when the
library or a CUDA device is missing, every solver entry point raises.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libcs_gb300.so")

CS_OK = 0
STATUS_NAMES = {0: "fresh", 1: "line-search", 2: "converged", 3: "done", 4: "failed", 5: "remesh"}

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)


class ModuleDesc(ctypes.Structure):
    _fields_ = [("problem_src", ctypes.c_char_p), ("ny", ctypes.c_int), ("nz", ctypes.c_int), ("np", ctypes.c_int),
                ("np_eff", ctypes.c_int), ("n_theta", ctypes.c_int), ("m", ctypes.c_int),
                ("lobatto_A", _dp), ("lobatto_b", _dp), ("lobatto_c", _dp), ("gauss_w", _dp), ("gauss_L", _dp),
                ("gauss_I", _dp), ("L0", _dp), ("L1", _dp), ("cache_dir", ctypes.c_char_p),
                ("layout", ctypes.c_int), ("precision", ctypes.c_int)]


class Opts(ctypes.Structure):
    _fields_ = [("tol", ctypes.c_double), ("max_iter", ctypes.c_int), ("max_mesh", ctypes.c_int),
                ("max_nodes", ctypes.c_int), ("min_nodes", ctypes.c_int), ("max_linesearch", ctypes.c_int),
                ("alpha0", ctypes.c_double), ("alpha_m", ctypes.c_double), ("beta", ctypes.c_double),
                ("check_every", ctypes.c_int), ("babd_path", ctypes.c_int), ("residual_type", ctypes.c_int),
                ("scale_by_time", ctypes.c_int), ("residual2", ctypes.c_int), ("refine", ctypes.c_int),
                ("ls_grow", ctypes.c_int)]


class Stats(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int), ("N", ctypes.c_int), ("newton_steps", ctypes.c_int),
                ("residual_evals", ctypes.c_int), ("segment_evals", ctypes.c_int), ("remeshes", ctypes.c_int),
                ("continuation_steps", ctypes.c_int), ("singular", ctypes.c_int), ("fail_reason", ctypes.c_int),
                ("alpha", ctypes.c_double), ("max_residual", ctypes.c_double), ("last_norm", ctypes.c_double)]


class Profile(ctypes.Structure):
    _fields_ = [("launches", ctypes.c_longlong), ("super_steps", ctypes.c_longlong),
                ("intervals_condensed", ctypes.c_longlong), ("systems_solved", ctypes.c_longlong),
                ("residual_intervals", ctypes.c_longlong), ("condense_launches", ctypes.c_longlong),
                ("babd_launches", ctypes.c_longlong), ("residual_launches", ctypes.c_longlong),
                ("condense_ms", ctypes.c_double), ("babd_ms", ctypes.c_double), ("residual_ms", ctypes.c_double)]


class TuneResult(ctypes.Structure):
    _fields_ = [("lanes", ctypes.c_int), ("block", ctypes.c_int), ("grid", ctypes.c_int), ("candidates", ctypes.c_int),
                ("ms", ctypes.c_double), ("default_ms", ctypes.c_double)]


# cs_progress_fn: void (*)(void* user, int active, long long super_steps)
PROGRESS_FN = ctypes.CFUNCTYPE(None, ctypes.c_void_p, ctypes.c_int, ctypes.c_longlong)


# every symbol declared in include/cs_gb300.h: name -> (restype, argtypes)
SIGNATURES = {
    "cs_module_load": (ctypes.c_int, [ctypes.POINTER(ModuleDesc), ctypes.POINTER(ctypes.c_void_p)]),
    "cs_module_free": (None, [ctypes.c_void_p]),
    "cs_opts_default": (None, [ctypes.POINTER(Opts)]),
    "cs_batch_create": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_longlong, ctypes.c_void_p,
                                       ctypes.POINTER(ctypes.c_void_p)]),
    "cs_batch_free": (None, [ctypes.c_void_p]),
    "cs_batch_set_guess": (ctypes.c_int, [ctypes.c_void_p, _ip, _dp, _dp, _dp, _dp, _dp]),
    "cs_batch_set_state": (ctypes.c_int, [ctypes.c_void_p, _ip, _dp, _dp, _dp, _dp, _dp, _dp]),
    "cs_solve": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(Opts)]),
    "cs_batch_set_progress": (ctypes.c_int, [ctypes.c_void_p, PROGRESS_FN, ctypes.c_void_p]),
    "cs_batch_sizes": (ctypes.c_int, [ctypes.c_void_p, _ip, ctypes.POINTER(ctypes.c_longlong)]),
    "cs_get_solution": (ctypes.c_int, [ctypes.c_void_p, _dp, _dp, _dp, _dp, ctypes.POINTER(Stats)]),
    "cs_stage_residual": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_double, _dp, _dp, _dp]),
    "cs_stage_newton_direction": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_double, _dp, _dp, _dp, _dp, _dp]),
    "cs_stage_segment_residual": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_double, ctypes.c_double, _dp, _dp]),
    "cs_stage_remesh": (ctypes.c_int, [ctypes.c_void_p, _dp, _ip]),
    "cs_get_state": (ctypes.c_int, [ctypes.c_void_p, _dp, _dp, _dp, _dp, _dp, _dp]),
    "cs_last_error": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_size_t]),
    "cs_time_condense": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, _dp]),
    "cs_measure_fp64_peak": (ctypes.c_int, [_dp]),
    "cs_measure_dmma_peak": (ctypes.c_int, [_dp]),
    "cs_profiler_start": (ctypes.c_int, []),
    "cs_batch_set_opts": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "cs_autotune_condense": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(TuneResult)]),
    "cs_profiler_stop": (ctypes.c_int, []),
    "cs_batch_reset": (ctypes.c_int, [ctypes.c_void_p]),
    "cs_profile_reset": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "cs_profile_get": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(Profile)]),
    "cs_pinned_alloc": (ctypes.c_void_p, [ctypes.c_size_t]),
    "cs_pinned_free": (None, [ctypes.c_void_p]),
    "cs_babd_solve": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int] + [ctypes.c_void_p] * 10 +
                      [ctypes.POINTER(ctypes.c_int), ctypes.c_void_p]),
    "cs_mlp_create": (ctypes.c_int, [ctypes.c_int] * 4 + [ctypes.c_ulonglong, ctypes.POINTER(ctypes.c_void_p)]),
    "cs_mlp_free": (None, [ctypes.c_void_p]),
    "cs_mlp_num_params": (ctypes.c_longlong, [ctypes.c_void_p]),
    "cs_mlp_set_normalization": (ctypes.c_int, [ctypes.c_void_p] + [ctypes.POINTER(ctypes.c_float)] * 4),
    "cs_mlp_get_params": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_float)]),
    "cs_mlp_set_params": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_float)]),
    "cs_mlp_gradient": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float),
                                       ctypes.c_int, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_float)]),
    "cs_mlp_train": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float),
                                    ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_float, ctypes.c_ulonglong,
                                    ctypes.POINTER(ctypes.c_double)]),
    "cs_mlp_predict": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_float), ctypes.c_int,
                                      ctypes.POINTER(ctypes.c_float)]),
    "cs_mlp_predict_device": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                                             ctypes.c_void_p]),
    "cs_batch_warm_start": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_int]),
    "cs_batch_set_spares": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int]),
    "cs_format_solutions": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_longlong, ctypes.c_void_p]),
    "cs_format_double": (ctypes.c_int, [ctypes.c_double, ctypes.c_char_p]),
    "cs_mlp_set_schedule": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_float]),
    "cs_device_alloc": (ctypes.c_void_p, [ctypes.c_size_t]),
    "cs_device_free": (None, [ctypes.c_void_p]),
    "cs_copy": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int]),
    "cs_tc_update": (ctypes.c_int, [ctypes.c_int] * 4 + [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_int,
                                                          ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]),
    "cs_babd_solve_noalloc": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int] + [ctypes.c_void_p] * 10 +
                              [ctypes.POINTER(ctypes.c_int), ctypes.c_void_p]),
}

_lib = None


class CsError(RuntimeError):
    pass


def load(path=LIB_PATH):
    """Load the library (no fallback: raises if it is missing)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise CsError("libcs_gb300.so not built (run __graft_entry__.build() or python -m build): %s" % path)
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def last_error():
    lib = load()
    buf = ctypes.create_string_buffer(8192)
    lib.cs_last_error(buf, len(buf))
    return buf.value.decode(errors="replace")


def check(rc, what):
    if rc != CS_OK:
        raise CsError("%s failed (code %d): %s" % (what, rc, last_error()))


def dptr(a):
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"], "arrays must be C-contiguous float64"
    return a.ctypes.data_as(_dp)


def fptr(a):
    if a is None:
        return None
    assert a.dtype == np.float32 and a.flags["C_CONTIGUOUS"], "arrays must be C-contiguous float32"
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


def iptr(a):
    if a is None:
        return None
    assert a.dtype == np.int32 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_ip)
