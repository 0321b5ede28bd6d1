"""Batched operators over many volumes (different N, trajectories, coils).

`NufftBatch([obj_1, ..., obj_n], [nc_1, ..., nc_n])` runs fNUFT, aNUFT and the
CG iNUFT of every volume with one kernel launch per stage (libnufft3d's
nufft3d_batch_*).  Each volume's result equals its own object's.  Objects
must be distinct plan handles (use ``obj.share()`` to repeat a trajectory)
with the same J, kernel type and 2-D/3-D.  Tensors are torch CUDA tensors in
the layouts of ``nufft_3d`` (images (nc, N3, N2, N1), samples (nc, M)).
The batched kernels read each volume's stored H but not its stored H' (the
batched spread evaluates the kernel), so objects made only for a batch can be
created with ``spread_table=0`` to save that memory.
"""
from __future__ import annotations

import ctypes

from . import _lib


class NufftBatch:
    def __init__(self, objs, ncs):
        if len(objs) != len(ncs) or not objs:
            raise ValueError("one coil count per volume")
        self.objs = list(objs)
        self.ncs = [int(c) for c in ncs]
        self._L = _lib.load()
        n = len(objs)
        plans = (ctypes.c_void_p * n)(*[o.plan.value if isinstance(o.plan, ctypes.c_void_p) else o.plan
                                        for o in objs])
        ncs_c = (ctypes.c_int * n)(*self.ncs)
        h = ctypes.c_void_p()
        _lib.check(self._L.nufft3d_batch_create(ctypes.cast(plans, ctypes.c_void_p),
                                                ctypes.cast(ncs_c, ctypes.c_void_p), n, ctypes.byref(h)))
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            self._L.nufft3d_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @staticmethod
    def _ptrs(ts):
        return (ctypes.c_void_p * len(ts))(*[t.data_ptr() for t in ts])

    @staticmethod
    def _stream(t):
        import torch
        return ctypes.c_void_p(torch.cuda.current_stream(t.device).cuda_stream)

    def _img(self, v, dev):
        import torch
        o = self.objs[v]
        return torch.empty((self.ncs[v],) + tuple(int(n) for n in o.N[::-1]), dtype=torch.complex64, device=dev)

    def forward(self, xs):
        import torch
        xs = [x.contiguous() for x in xs]
        ks = [torch.empty((self.ncs[v], self.objs[v].M), dtype=torch.complex64, device=xs[v].device)
              for v in range(len(xs))]
        _lib.check(self._L.nufft3d_batch_forward(self._h, self._ptrs(xs), self._ptrs(ks), self._stream(xs[0])))
        return ks

    def adjoint(self, ks):
        ks = [k.contiguous() for k in ks]
        xs = [self._img(v, ks[v].device) for v in range(len(ks))]
        _lib.check(self._L.nufft3d_batch_adjoint(self._h, self._ptrs(ks), self._ptrs(xs), self._stream(ks[0])))
        return xs

    def inverse(self, raws, maxit=20, damp=0.0, tol=0.0, return_iters=False):
        """CG iNUFT of every (volume, coil) system, W = d (iNUFT.m default path)."""
        raws = [r.contiguous() for r in raws]
        xs = [self._img(v, raws[v].device) for v in range(len(raws))]
        its = (ctypes.c_int * sum(self.ncs))()
        _lib.check(self._L.nufft3d_batch_inverse(self._h, self._ptrs(raws), self._ptrs(xs), int(maxit), float(damp),
                                                 float(tol), ctypes.cast(its, ctypes.c_void_p), self._stream(raws[0])))
        return (xs, list(its)) if return_iters else xs
