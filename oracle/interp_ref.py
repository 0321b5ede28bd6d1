"""ctypes front end of the matrix-free FP64 interpolation oracle (interp_ref.c).

TEST INFRASTRUCTURE ONLY (see nufft_ref.py).  The shared object is built by
``oracle/build_oracle.sh`` (called from ``__graft_entry__.build()``); if it is
missing this module builds it on first use, since gcc exists wherever the
tests run.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_SO = os.path.join(_HERE, "_build", "liboracle_interp.so")
_lib = None


def build(force=False):
    if force or not os.path.exists(_SO):
        subprocess.check_call(["bash", os.path.join(_HERE, "build_oracle.sh")])
    return _SO


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_SO)
        args = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
                ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.c_int,
                ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
        for name in ("oracle_interp_forward", "oracle_interp_adjoint"):
            f = getattr(L, name)
            f.argtypes = args
            f.restype = None
        _lib = L
    return _lib


def _common(ref):
    om_g = np.ascontiguousarray(ref.om_g.T, dtype=np.float64)  # (M, 3) == [3 x M] col-major
    ok = np.ascontiguousarray(ref.ok, dtype=np.uint8)
    K = np.ascontiguousarray(ref.K, dtype=np.int64)
    return om_g, ok, K


def interp_forward(ref, grid):
    """y = H * grid; grid (prod(K),) or (prod(K), nc) -> (M,) or (M, nc) complex128."""
    g = np.asarray(grid)
    squeeze = g.ndim == 1
    g = g.reshape(g.shape[0], -1)
    nc = g.shape[1]
    gc = np.asfortranarray(g.astype(np.complex128))
    out = np.zeros((ref.M, nc), dtype=np.complex128, order="F")
    om_g, ok, K = _common(ref)
    lib().oracle_interp_forward(om_g.ctypes.data, ok.ctypes.data, ref.M, K.ctypes.data,
                                ref.J, ref.alpha, int(ref.radial), int(ref.N[2] == 1),
                                gc.ctypes.data, nc, out.ctypes.data)
    if not np.iscomplexobj(grid):
        out = out.real.copy()
    return out[:, 0] if squeeze else out


def interp_adjoint(ref, y):
    """grid = H' * y; y (M,) or (M, nc) -> (prod(K),) or (prod(K), nc)."""
    yy = np.asarray(y)
    squeeze = yy.ndim == 1
    yy = yy.reshape(ref.M, -1)
    nc = yy.shape[1]
    yc = np.asfortranarray(yy.astype(np.complex128))
    G = int(np.prod(ref.K))
    grid = np.zeros((G, nc), dtype=np.complex128, order="F")
    om_g, ok, K = _common(ref)
    lib().oracle_interp_adjoint(om_g.ctypes.data, ok.ctypes.data, ref.M, K.ctypes.data,
                                ref.J, ref.alpha, int(ref.radial), int(ref.N[2] == 1),
                                yc.ctypes.data, nc, grid.ctypes.data)
    if not np.iscomplexobj(y):
        grid = grid.real.copy()
    return grid[:, 0] if squeeze else grid
