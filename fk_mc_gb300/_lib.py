"""ctypes binding of libfkg.so (the C ABI declared in include/fkg.h).

The product path has no CPU fallback: if the CUDA library is missing or a
call fails, an exception is raised.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libfkg.so")

FKG_OK = 0
FKG_ERR = {-1: "FKG_ERR_ARG", -2: "FKG_ERR_CUDA", -3: "FKG_ERR_ALLOC", -4: "FKG_ERR_STATE",
           -5: "FKG_ERR_TIMEOUT", -6: "FKG_ERR_NUMERIC"}
PREC = {"f64": 0, "mixed": 1}
METHOD = {"ed": 0, "chebyshev": 1}

# every symbol include/fkg.h declares, with its ctypes signature
_i32p = ctypes.POINTER(ctypes.c_int32)
_dp = ctypes.POINTER(ctypes.c_double)
_vp = ctypes.c_void_p
SIGNATURES = {
    "fkg_create": ([ctypes.c_int, ctypes.c_int, ctypes.c_uint], _vp),
    "fkg_destroy": ([_vp], None),
    "fkg_last_error": ([_vp], ctypes.c_char_p),
    "fkg_set_precision": ([_vp, ctypes.c_int], ctypes.c_int),
    "fkg_set_hopping": ([_vp, ctypes.c_int, ctypes.c_int, _i32p, _i32p, _dp], ctypes.c_int),
    "fkg_eigh_logz": ([_vp, ctypes.c_int, _i32p, _dp, _dp, _dp, _dp, _dp, _dp, _dp], ctypes.c_int),
    "fkg_set_chebyshev": ([_vp, ctypes.c_int, ctypes.c_int], ctypes.c_int),
    "fkg_chebyshev_logz": ([_vp, ctypes.c_int, _i32p, _dp, _dp, _dp, _dp, _dp, _dp, _i32p], ctypes.c_int),
    "fkg_set_method": ([_vp, ctypes.c_int], ctypes.c_int),
    "fkg_rank1_logz": ([_vp, ctypes.c_int, ctypes.c_int, _dp, _dp, _dp, _dp, _dp, _dp], ctypes.c_int),
    "fkg_rank1_logz_device": ([_vp, ctypes.c_int, ctypes.c_int, _vp, _vp, _vp, _vp, _vp, _vp], ctypes.c_int),
    "fkg_chains_init": ([_vp, ctypes.c_int, _i32p, _i32p, _dp, _dp, _dp, _dp], ctypes.c_int),
    "fkg_propose_accept": ([_vp, ctypes.c_int, _i32p, _dp, _i32p, _dp], ctypes.c_int),
    "fkg_propose_accept_device": ([_vp, ctypes.c_int, _vp, _vp, _vp, _vp], ctypes.c_int),
    "fkg_chains_get": ([_vp, _i32p, _dp, _dp], ctypes.c_int),
    "fkg_free_energy_grad": ([_vp, ctypes.c_int, _i32p, _i32p, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp],
                             ctypes.c_int),
    "fkg_set_stiffness_ops": ([_vp, ctypes.c_int, ctypes.c_int, _i32p, _i32p, _dp, _dp], ctypes.c_int),
    "fkg_measure_ipr": ([_vp, ctypes.c_int, _i32p, _dp, _dp, _dp], ctypes.c_int),
    "fkg_measure_stiffness": ([_vp, ctypes.c_int, _i32p, _dp, _dp, _dp, ctypes.c_int, _dp, ctypes.c_double, _dp],
                              ctypes.c_int),
    "fkg_launch_count": ([_vp], ctypes.c_longlong),
    "fkg_set_stream": ([_vp, _vp], ctypes.c_int),
    "fkg_set_tuning": ([_vp, ctypes.c_int, ctypes.c_int, ctypes.c_int], ctypes.c_int),
    "fkg_set_tuning_back": ([_vp, ctypes.c_int, ctypes.c_int], ctypes.c_int),
    "fkg_set_graphs": ([_vp, ctypes.c_int], ctypes.c_int),
    "fkg_set_wait_limit": ([_vp, ctypes.c_longlong], ctypes.c_int),
    "fkg_profile": ([_vp, ctypes.c_int], ctypes.c_int),
    "fkg_stage_time": ([_vp, ctypes.c_int, _dp, ctypes.POINTER(ctypes.c_longlong)], ctypes.c_int),
    "fkg_eigh_logz_noalloc": ([ctypes.c_int, ctypes.c_int, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp,
                               ctypes.c_char_p, ctypes.c_int], ctypes.c_int),
}
STAGES = {"reduce": 0, "trieig": 1, "back": 2, "refine": 3, "logz": 4}

_lib = None


class FkgError(RuntimeError):
    pass


def load(path=LIB_PATH):
    """Load libfkg.so and bind every entry point. Raises if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise FkgError(f"CUDA library {path} is missing: run __graft_entry__.build() first")
    lib = ctypes.CDLL(path)
    for name, (args, res) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    _lib = lib
    return lib


def ptr(a, ctype):
    if a is None:
        return None
    return a.ctypes.data_as(ctypes.POINTER(ctype))


def i32(a):
    return ptr(a, ctypes.c_int32)


def f64(a):
    return ptr(a, ctypes.c_double)


def check(ctx, rc, what):
    if rc != FKG_OK:
        msg = load().fkg_last_error(ctx)
        raise FkgError(f"{what} failed with {FKG_ERR.get(rc, rc)}: {msg.decode() if msg else ''}")


def as_i32(x):
    return np.ascontiguousarray(x, dtype=np.int32)


def as_f64(x):
    return np.ascontiguousarray(x, dtype=np.float64)
