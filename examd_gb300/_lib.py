"""Loader of the CUDA library (examd_gb300/_lib/libexamd_gb300.so) with ctypes prototypes.

The product has no CPU fallback: if the shared object is missing this module
raises, naming the build command.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libexamd_gb300.so")
# the index-checked build (python -m examd_gb300.build --checked), loaded instead when EXAMD_CHECKED=1
LIB_CHECKED_PATH = os.path.join(HERE, "_lib", "libexamd_gb300_checked.so")

MAX_TYPES = 4
STATIC_MAX_ATOMS = 1048576  # EXAMD_STATIC_MAX_ATOMS
STATIC_MAX_BOXES = 4096     # EXAMD_STATIC_MAX_BOXES
FP64 = 0
MIXED = 1

OK = 0
ERR_OUTSIDE = 109
ERR_ARG = 201
ERR_NB_TOO_SMALL = 202
ERR_CELL_OVERFLOW = 203
ERR_NONFINITE = 204
ERR_TIMEOUT = 205
ERR_CUDA = 206
ERR_NOMEM = 207
ERR_STATE = 208
ERR_NO_DEVICE = 209
ERR_IO = 210
ERR_PAIRFN = 211
ERR_CHECK = 212
POT_LJ, POT_LJ_SHIFTED, POT_WCA = 0, 1, 2


class Params(C.Structure):
    _fields_ = [
        ("precision", C.c_int),
        ("ntypes", C.c_int),
        ("eps", C.c_double * (MAX_TYPES * MAX_TYPES)),
        ("sigma", C.c_double * (MAX_TYPES * MAX_TYPES)),
        ("rc", C.c_double * (MAX_TYPES * MAX_TYPES)),
        ("mass", C.c_double * MAX_TYPES),
        ("cell_edge", C.c_double),
        ("tile", C.c_int * 3),
        ("warps", C.c_int),
        ("strict_box", C.c_int),
        ("device", C.c_int),
        ("potential", C.c_int),
        ("pair_tables", C.c_int),
        ("tile_balance", C.c_int),
        ("pair_skin", C.c_double),
        ("pair_list_capacity", C.c_int),
    ]


class Box(C.Structure):
    _fields_ = [("L", C.c_double * 3), ("natoms", C.c_int64)]


class Stats(C.Structure):
    _fields_ = [("epot", C.c_double), ("virial", C.c_double), ("ekin", C.c_double), ("steps", C.c_int64),
                ("ms", C.c_double)]


_lock = threading.Lock()
_lib = None


def load():
    """Load the library (once).  Raises FileNotFoundError if it was not built."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        checked = os.environ.get("EXAMD_CHECKED") == "1"
        path = LIB_CHECKED_PATH if checked else LIB_PATH
        if not os.path.exists(path):
            raise FileNotFoundError(
                f"{path} is missing: build it with `python -m examd_gb300.build{' --checked' if checked else ''}` "
                "(or __graft_entry__.build()); there is no CPU fallback")
        L = C.CDLL(path)
        dp = C.POINTER(C.c_double)
        ip = C.POINTER(C.c_int)
        i64p = C.POINTER(C.c_int64)
        vp = C.c_void_p
        ctxp = C.c_void_p
        sig = {
            "examd_default_params": (None, [C.POINTER(Params)]),
            "examd_gpu_create": (C.c_int, [C.POINTER(Params), C.c_int, C.POINTER(Box), C.POINTER(ctxp)]),
            "examd_gpu_destroy": (None, [ctxp]),
            "examd_gpu_set_atoms": (C.c_int, [ctxp, C.c_int64, dp, ip, dp]),
            "examd_gpu_forces": (C.c_int, [ctxp, dp, dp, dp, C.c_int]),
            "examd_gpu_forces_at": (C.c_int, [ctxp, dp, dp, dp, dp, C.c_int]),
            "examd_gpu_run": (C.c_int, [ctxp, C.c_int, C.c_double, C.c_int, dp, C.POINTER(Stats)]),
            "examd_gpu_prepare_run": (C.c_int, [ctxp, C.c_double, C.c_int, C.c_int]),
            "examd_gpu_time_phases": (C.c_int, [ctxp, C.c_int, C.c_double, dp]),
            "examd_gpu_list_info": (C.c_int, [ctxp, i64p, ip, ip, ip]),
            "examd_gpu_time_rebuild": (C.c_int, [ctxp, C.c_int, dp]),
            "examd_gpu_get_state": (C.c_int, [ctxp, dp, dp]),
            "examd_gpu_kinetic": (C.c_int, [ctxp, dp]),
            "examd_kinetic_static": (C.c_int, [C.c_int, C.c_int64, C.c_int, i64p, vp, vp, vp, vp, C.c_int, dp, dp,
                                               vp, C.c_char_p, C.c_int]),
            "examd_gpu_scale_velocities": (C.c_int, [ctxp, dp]),
            "examd_gpu_time_forces": (C.c_int, [ctxp, C.c_int, dp, dp]),
            "examd_autotune": (C.c_int, [C.POINTER(Params), C.c_int, C.POINTER(Box), C.c_int64, dp, ip, C.c_char_p,
                                         C.POINTER(Params), dp]),
            "examd_gpu_counters": (C.c_int, [ctxp, i64p, i64p, i64p, i64p, i64p]),
            "examd_gpu_strerror": (C.c_char_p, [C.c_int]),
            "examd_gpu_last_error": (C.c_char_p, [ctxp]),
            "examd_own_table": (C.c_int, [C.POINTER(C.c_byte), C.POINTER(C.c_ubyte)]),
            "examd_tile_split": (C.c_int, [C.c_int, C.c_double, C.c_int, C.c_int, C.POINTER(C.c_int),
                                           C.POINTER(C.c_int)]),
            "examd_host_alloc": (C.c_int, [C.POINTER(vp), C.c_int64]),
            "examd_host_free": (C.c_int, [vp]),
            "examd_read_particles": (C.c_int, [C.c_char_p, i64p, dp, dp, C.c_int64]),
            "examd_write_particles": (C.c_int, [C.c_char_p, C.c_int64, dp, dp]),
            "examd_gen_fcc": (C.c_int, [C.c_int, C.c_double, dp, dp]),
            "examd_gen_velocities": (C.c_int, [C.c_int64, ip, dp, C.c_double, C.c_uint64, dp]),
            "examd_gen_random": (C.c_int, [C.c_int64, C.c_int64, dp, dp, dp, C.c_double, C.c_uint64, C.c_int64,
                                           dp]),
            "examd_gen_jittered_sc": (C.c_int, [C.c_int, C.c_double, C.c_double, C.c_double, C.c_uint64, dp, ip,
                                                dp]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
        return L


class ExamdError(RuntimeError):
    def __init__(self, code: int, where: str = "", detail: str = ""):
        lib = _lib
        msg = lib.examd_gpu_strerror(code).decode() if lib is not None else str(code)
        super().__init__(f"{where}: examd status {code} ({msg}){' ' + detail if detail else ''}")
        self.code = code


def check(code: int, where: str = "", ctx=None, detail: str = ""):
    if code != OK:
        if ctx is not None and _lib is not None:
            detail = (_lib.examd_gpu_last_error(ctx) or b"").decode()
        raise ExamdError(code, where, detail)
