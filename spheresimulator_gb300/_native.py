"""ctypes binding of libsmob.so (the CUDA library). No CPU fallback exists: if the library
cannot be built or loaded, or no GPU is present, every call raises."""
import ctypes
import os

import numpy as np

from . import _build

SMOB_OK = 0
SMOB_ERR_ARG = 1
SMOB_ERR_CUDA = 2
SMOB_ERR_NOMEM = 3
SMOB_ERR_NOT_CONVERGED = 4
SMOB_ERR_NONFINITE = 5
SMOB_ERR_STATE = 6
SMOB_ERR_NO_DEVICE = 7

PREC_FP64 = 0
PREC_MIXED = 1
PREC_FLOAT_FLOAT = 2

STATUS_NAMES = {0: "OK", 1: "ARG", 2: "CUDA", 3: "NOMEM", 4: "NOT_CONVERGED", 5: "NONFINITE", 6: "STATE",
                7: "NO_DEVICE"}


class SmobError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("smob error %s (%d): %s" % (STATUS_NAMES.get(code, "?"), code, msg))
        self.code = code


class Geometry(ctypes.Structure):
    _fields_ = [("n_spheres", ctypes.c_int), ("centers", ctypes.POINTER(ctypes.c_double)),
                ("radii", ctypes.POINTER(ctypes.c_double)), ("quats", ctypes.POINTER(ctypes.c_double)),
                ("orders", ctypes.POINTER(ctypes.c_int)), ("problem", ctypes.POINTER(ctypes.c_int)),
                ("viscosity", ctypes.c_double)]


class SolveOpts(ctypes.Structure):
    _fields_ = [("tol", ctypes.c_double), ("restart", ctypes.c_int), ("max_iters", ctypes.c_int),
                ("precision", ctypes.c_int), ("warm_start", ctypes.c_int), ("inner_tol", ctypes.c_double),
                ("precond", ctypes.c_int)]


class ProblemStats(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int), ("iterations", ctypes.c_int), ("refinements", ctypes.c_int),
                ("operator_passes_fp64", ctypes.c_int), ("operator_passes_fp32", ctypes.c_int),
                ("relres", ctypes.c_double), ("bnorm", ctypes.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class ServerOpts(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int), ("max_slots", ctypes.c_int), ("hbm_budget_bytes", ctypes.c_double),
                ("restart", ctypes.c_int), ("max_iters", ctypes.c_int), ("precision", ctypes.c_int),
                ("inner_tol", ctypes.c_double), ("graphs", ctypes.c_int)]


class RequestInfo(ctypes.Structure):
    _fields_ = [("state", ctypes.c_int), ("status", ctypes.c_int), ("t_submit", ctypes.c_double),
                ("t_admit", ctypes.c_double), ("t_done", ctypes.c_double), ("bytes", ctypes.c_double),
                ("stats", ProblemStats), ("t_ctx", ctypes.c_double),
                ("route", ctypes.c_int)]


class ServerInfo(ctypes.Structure):
    _fields_ = [("queued", ctypes.c_int), ("running", ctypes.c_int), ("completed", ctypes.c_longlong),
                ("bytes_in_use", ctypes.c_double), ("peak_bytes", ctypes.c_double), ("budget_bytes", ctypes.c_double),
                ("uptime_s", ctypes.c_double), ("peak_running", ctypes.c_int)]


_lib = None
_DP = ctypes.POINTER(ctypes.c_double)
_IP = ctypes.POINTER(ctypes.c_int)
_VP = ctypes.c_void_p


def library_path():
    return _build.LIB


def lib():
    """Load (building first if stale) libsmob.so."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.build()
    L = ctypes.CDLL(path)
    S = ctypes.c_int
    sig = {
        "smob_create": (S, [ctypes.POINTER(_VP), ctypes.POINTER(Geometry), ctypes.c_int]),
        "smob_destroy": (S, [_VP]),
        "smob_last_error": (ctypes.c_char_p, []),
        "smob_version": (S, [_IP, _IP]),
        "smob_get_sizes": (S, [_VP, _IP, _IP, _IP, _IP]),
        "smob_get_grid": (S, [_VP, _DP, _DP, _DP]),
        "smob_get_near_pairs": (S, [_VP, _IP, _IP]),
        "smob_apply": (S, [_VP, _DP, _DP, ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_int]),
        "smob_apply_p2p": (S, [_VP, _DP, _DP, ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_int]),
        "smob_apply_lop": (S, [_VP, _DP, _DP, ctypes.c_double]),
        "smob_project_null_space": (S, [_VP, _DP]),
        "smob_far_field": (S, [_VP, _DP, _DP, ctypes.c_double, ctypes.c_double, ctypes.c_int]),
        "smob_near_field": (S, [_VP, _DP, _DP, ctypes.c_double, ctypes.c_double, ctypes.c_int]),
        "smob_sh_g2s": (S, [_VP, _DP, _DP]),
        "smob_sh_s2g": (S, [_VP, _DP, _DP]),
        "smob_coeff_offsets": (S, [_VP, _IP]),
        "smob_solve_mob": (S, [_VP, _DP, _DP, _DP, ctypes.POINTER(SolveOpts), ctypes.POINTER(ProblemStats)]),
        "smob_solve_mob_device": (S, [_VP, _VP, _VP, _VP, ctypes.POINTER(SolveOpts), ctypes.POINTER(ProblemStats)]),
        "smob_mob_apply": (S, [_VP, _DP, _DP, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                               ctypes.POINTER(SolveOpts)]),
        "smob_solve_mob_multi": (S, [_VP, ctypes.c_int, _DP, _DP, _DP, ctypes.POINTER(SolveOpts),
                                     ctypes.POINTER(ProblemStats)]),
        "smob_write_vtu": (S, [_VP, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p, _DP]),
        "smob_write_xyz": (S, [_VP, ctypes.c_char_p, _IP, ctypes.c_double]),
        "smob_step_euler": (S, [_VP, _DP, ctypes.c_double]),
        "smob_step_euler_device": (S, [_VP, _VP, ctypes.c_double]),
        "smob_set_geometry": (S, [_VP, _DP, _DP]),
        "smob_get_geometry": (S, [_VP, _DP, _DP]),
        "smob_device_alloc": (S, [_VP, ctypes.c_size_t, ctypes.POINTER(_VP)]),
        "smob_device_free": (S, [_VP, _VP]),
        "smob_memcpy_h2d": (S, [_VP, _VP, _VP, ctypes.c_size_t]),
        "smob_memcpy_d2h": (S, [_VP, _VP, _VP, ctypes.c_size_t]),
        "smob_synchronize": (S, [_VP]),
        "smob_profile_enable": (S, [_VP, ctypes.c_int]),
        "smob_profile_count": (S, [_VP, _IP]),
        "smob_profile_get": (S, [_VP, ctypes.c_int, ctypes.c_char_p, ctypes.c_int, ctypes.POINTER(ctypes.c_longlong),
                                 _DP]),
        "smob_profile_reset": (S, [_VP]),
        "smob_launch_count": (S, [_VP, ctypes.POINTER(ctypes.c_longlong)]),
        "smob_tuning": (S, [_VP, _IP, _DP, _IP]),
        "smob_set_graphs": (S, [_VP, ctypes.c_int]),
        "smob_set_loop_graph": (S, [_VP, ctypes.c_int]),
        "smob_warm_orders": (S, [ctypes.POINTER(ctypes.c_int), ctypes.c_int]),
        "smob_loop_graph_info": (S, [_VP, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]),
        "smob_launch_stats": (S, [_VP, ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_longlong)]),
        "smob_set_far_tile": (S, [_VP, ctypes.c_int]),
        "smob_set_near_tc": (S, [_VP, ctypes.c_int]),
        "smob_set_coarse_tc": (S, [_VP, ctypes.c_int]),
        "smob_set_multi_shared_pairs": (S, [_VP, ctypes.c_int]),
        "smob_coarse_tc_info": (S, [_VP, ctypes.POINTER(ctypes.c_int)]),
        "smob_set_sphere_tc": (S, [_VP, ctypes.c_int]),
        "smob_tc_info": (S, [_VP, _IP, _IP]),
        "smob_recycle_info": (S, [_VP, _IP, _IP]),
        "smob_set_far_compression": (S, [_VP, ctypes.c_double, ctypes.c_double]),
        "smob_set_far_coarse_targets": (S, [_VP, ctypes.c_int]),
        "smob_far_compression_info": (S, [_VP, ctypes.c_int, _DP, _IP, _IP]),
        "smob_far_pairs": (S, [_VP, ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_longlong),
                               ctypes.POINTER(ctypes.c_longlong)]),
        "smob_far_pairs_set": (S, [_VP, ctypes.c_int, ctypes.POINTER(ctypes.c_longlong),
                                   ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_longlong)]),
        "smob_recycle_clear": (S, [_VP]),
        "smob_timer_mark": (S, [_VP]),
        "smob_timer_elapsed": (S, [_VP, _DP]),
        "smob_flush_l2": (S, [_VP, ctypes.c_size_t]),
        "smob_measure_fma_peaks": (S, [ctypes.c_int, _DP, _DP]),
        "smob_far_traction_noalloc": (S, [_VP, _VP, _VP, _VP, _VP, ctypes.c_int, ctypes.c_double, _VP, _VP]),
        "smob_server_create": (S, [ctypes.POINTER(_VP), ctypes.POINTER(ServerOpts)]),
        "smob_server_submit": (S, [_VP, ctypes.POINTER(Geometry), _DP, ctypes.c_double,
                                   ctypes.POINTER(ctypes.c_longlong)]),
        "smob_server_poll": (S, [_VP, ctypes.c_longlong, _DP, ctypes.POINTER(RequestInfo), _IP]),
        "smob_server_wait": (S, [_VP, ctypes.c_longlong, ctypes.c_double, _DP, ctypes.POINTER(RequestInfo)]),
        "smob_server_release": (S, [_VP, ctypes.c_longlong]),
        "smob_server_stats": (S, [_VP, ctypes.POINTER(ServerInfo)]),
        "smob_server_destroy": (S, [_VP]),
        "smob_server_partition": (S, [_VP, ctypes.c_int]),
        "smob_server_partition_info": (S, [_VP, _IP, _IP]),
        "smob_request_bytes": (ctypes.c_size_t, [ctypes.c_int, _IP, ctypes.c_int]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def exported_symbols():
    """Names of the entry points declared in include/smob.h that the binding resolves."""
    return [n for n in dir(lib()) if n.startswith("smob_")]


def check(code, allow=()):
    if code != SMOB_OK and code not in allow:
        raise SmobError(code, lib().smob_last_error().decode(errors="replace"))
    return code


def dptr(a):
    return None if a is None else a.ctypes.data_as(_DP)


def iptr(a):
    return None if a is None else a.ctypes.data_as(_IP)


def f64(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.float64)


def i32(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.int32)
