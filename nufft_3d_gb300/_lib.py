"""ctypes binding of libnufft3d.so (the C ABI declared in include/nufft3d.h).

The library is the only compute path: if it is missing this module raises
immediately -- there is no CPU or PyTorch fallback.
"""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libnufft3d.so")

SUCCESS = 0
ERR_ARG = -1
ERR_SIZE = -2
ERR_CUDA = -3
ERR_NOMEM = -4
ERR_UNSUPPORTED = -5
ERR_TIMEOUT = -6
SOLVER_MINRES = 0
SOLVER_CG = 1

_ERR_NAMES = {ERR_ARG: "NUFFT3D_ERR_ARG", ERR_SIZE: "NUFFT3D_ERR_SIZE", ERR_CUDA: "NUFFT3D_ERR_CUDA",
              ERR_NOMEM: "NUFFT3D_ERR_NOMEM", ERR_UNSUPPORTED: "NUFFT3D_ERR_UNSUPPORTED",
              ERR_TIMEOUT: "NUFFT3D_ERR_TIMEOUT"}


class NufftError(RuntimeError):
    """A libnufft3d call returned a negative status."""

    def __init__(self, code, msg):
        super().__init__("%s (%d): %s" % (_ERR_NAMES.get(code, "error"), code, msg))
        self.code = code


class Opts(ctypes.Structure):
    _fields_ = [("J", ctypes.c_double), ("u", ctypes.c_double), ("alpha", ctypes.c_double),
                ("radial", ctypes.c_int), ("gpu", ctypes.c_int), ("device", ctypes.c_int),
                ("d", ctypes.c_void_p), ("density_iters", ctypes.c_int),
                ("tile", ctypes.c_int * 3), ("max_coils_per_pass", ctypes.c_int),
                ("max_samples_per_block", ctypes.c_int), ("verbose", ctypes.c_int),
                ("tap_table", ctypes.c_int), ("wait_polls", ctypes.c_int), ("spread_table", ctypes.c_int)]


class Info(ctypes.Structure):
    _fields_ = [("N", ctypes.c_int32 * 3), ("K", ctypes.c_int32 * 3), ("M", ctypes.c_int64),
                ("nnz", ctypes.c_int64), ("J", ctypes.c_double), ("u", ctypes.c_double),
                ("alpha", ctypes.c_double), ("radial", ctypes.c_int), ("tile", ctypes.c_int * 3),
                ("n_blocks", ctypes.c_int64), ("taps_per_sample", ctypes.c_double),
                ("device_bytes", ctypes.c_int64), ("tap_table_bytes", ctypes.c_int64),
                ("kernel_polynomial", ctypes.c_int), ("spread_table_bytes", ctypes.c_int64)]


class TuneResult(ctypes.Structure):
    _fields_ = [("samples_per_block", ctypes.c_int), ("coils_per_pass", ctypes.c_int),
                ("ms_best", ctypes.c_double), ("ms_default", ctypes.c_double), ("candidates", ctypes.c_int),
                ("from_cache", ctypes.c_int)]


# name -> (restype, argtypes); the exported surface of include/nufft3d.h
_P = ctypes.c_void_p
SIGNATURES = {
    "nufft3d_opts_default": (ctypes.c_int, [ctypes.POINTER(Opts)]),
    "nufft3d_plan_create": (ctypes.c_int, [_P, ctypes.c_int64, _P, ctypes.c_int, ctypes.POINTER(Opts),
                                           ctypes.POINTER(ctypes.c_void_p)]),
    "nufft3d_plan_destroy": (ctypes.c_int, [_P]),
    "nufft3d_plan_share": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_void_p)]),
    "nufft3d_plan_set_sms": (ctypes.c_int, [_P, ctypes.c_int]),
    "nufft3d_plan_set_host_copy": (ctypes.c_int, [_P, ctypes.c_int]),
    "nufft3d_plan_tune": (ctypes.c_int, [_P, ctypes.c_int, ctypes.c_int, ctypes.POINTER(TuneResult)]),
    "nufft3d_plan_footprint": (ctypes.c_int, [_P, ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_int64)]),
    "nufft3d_plan_info": (ctypes.c_int, [_P, ctypes.POINTER(Info)]),
    "nufft3d_get_deap": (ctypes.c_int, [_P, _P]),
    "nufft3d_get_density": (ctypes.c_int, [_P, _P]),
    "nufft3d_forward": (ctypes.c_int, [_P, _P, _P, ctypes.c_int, _P]),
    "nufft3d_adjoint": (ctypes.c_int, [_P, _P, _P, ctypes.c_int, _P]),
    "nufft3d_normal": (ctypes.c_int, [_P, _P, _P, ctypes.c_int, ctypes.c_double, _P, _P]),
    "nufft3d_forward_noalloc": (ctypes.c_int, [_P, _P, _P, ctypes.c_int, _P]),
    "nufft3d_forward_noalloc_scratch_bytes": (ctypes.c_size_t, []),
    "nufft3d_forward_host": (ctypes.c_int, [_P, _P, _P, ctypes.c_int]),
    "nufft3d_adjoint_host": (ctypes.c_int, [_P, _P, _P, ctypes.c_int]),
    "nufft3d_inverse": (ctypes.c_int, [_P, _P, _P, ctypes.c_int, ctypes.c_int, ctypes.c_double, _P,
                                       ctypes.c_int, ctypes.c_double, _P, _P]),
    "nufft3d_inverse_host": (ctypes.c_int, [_P, _P, _P, ctypes.c_int, ctypes.c_int, ctypes.c_double, _P,
                                            ctypes.c_int, ctypes.c_double, _P]),
    "nufft3d_inverse_phase": (ctypes.c_int, [_P, _P, _P, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                             ctypes.c_double, _P, ctypes.c_double, _P, _P]),
    "nufft3d_inverse_phase_host": (ctypes.c_int, [_P, _P, _P, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                                  ctypes.c_double, _P, ctypes.c_double, _P]),
    "nufft3d_inverse_x0": (ctypes.c_int, [_P, _P, _P, ctypes.c_int, ctypes.c_int, ctypes.c_double, _P,
                                          ctypes.c_int, ctypes.c_double, _P, _P]),
    "nufft3d_inverse_x0_host": (ctypes.c_int, [_P, _P, _P, ctypes.c_int, ctypes.c_int, ctypes.c_double, _P,
                                               ctypes.c_int, ctypes.c_double, _P]),
    "nufft3d_density": (ctypes.c_int, [_P, ctypes.c_int]),
    "nufft3d_batch_create": (ctypes.c_int, [_P, _P, ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)]),
    "nufft3d_batch_destroy": (ctypes.c_int, [_P]),
    "nufft3d_batch_forward": (ctypes.c_int, [_P, _P, _P, _P]),
    "nufft3d_batch_adjoint": (ctypes.c_int, [_P, _P, _P, _P]),
    "nufft3d_batch_inverse": (ctypes.c_int, [_P, _P, _P, ctypes.c_int, ctypes.c_double, ctypes.c_double, _P, _P]),
    "nufft3d_check_status": (ctypes.c_int, [_P, _P]),
    "nufft3d_kernel_eval": (ctypes.c_int, [_P, _P, _P, ctypes.c_int64, _P]),
    "nufft3d_profile": (ctypes.c_int, [_P, ctypes.c_int]),
    "nufft3d_profile_read": (ctypes.c_int, [_P, ctypes.c_char_p, ctypes.c_int]),
    "nufft3d_last_error": (ctypes.c_char_p, []),
    "nufft3d_version": (ctypes.c_char_p, []),
}

_lib = None


def load(path=None):
    """Load libnufft3d.so (raises if it has not been built)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise ImportError("libnufft3d.so not found at %s: run `python -c \"import __graft_entry__ as g; "
                          "g.build()\"` (or nufft_3d_gb300/build.py) first" % p)
    L = ctypes.CDLL(p)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    if path is None:
        _lib = L
    return L


def last_error():
    return load().nufft3d_last_error().decode()


def check(status):
    if status != SUCCESS:
        raise NufftError(status, last_error())
    return status
