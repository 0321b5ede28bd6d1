"""Host-side drop-in of the MATLAB ``@nufft_3d`` class, over libnufft3d.so.

Mirrors the reference interface (paths relative to the reference project):

* ``nufft_3d(om, N, 'J', 6, 'u', 2, ...)``      @nufft_3d/nufft_3d.m:54-251
  (name/value pairs positionally or as keywords; same defaults J=4, u=2,
  alpha=0 -> Beatty, radial=1, gpu=1; same error conditions).
* ``obj.fNUFT(x)``  / ``obj.aNUFT(k)``           @nufft_3d/fNUFT.m, aNUFT.m
* ``obj.iNUFT(raw, maxit, damp, W)``             @nufft_3d/iNUFT.m:2-138
* ``obj.discrep(data, stddev)``                  @nufft_3d/discrep.m:2-69
* ``obj * x`` / ``obj.ctranspose() * y``         (mtimes: fNUFT / aNUFT)
* properties J, u, N, alpha, radial, gpu, K, U, d, nnz (nufft_3d.m:26-43);
  ``H``/``HT`` do not exist -- the interpolation is matrix-free.

Arrays: numpy inputs are read in MATLAB column-major order -- images
(N1, N2, N3[, nc]), samples (M[, nc]) or (nr, ny[, nc]) -- and results come
back the same way (complex64).  torch CUDA tensors stay on the device: their
memory is read as the same column-major layout, i.e. C-contiguous tensors of
shape (nc, N3, N2, N1) for images and (nc, M) for samples.
"""
from __future__ import annotations

import ctypes
import math

import numpy as np

from . import _lib

_PROPS = ("J", "u", "alpha", "radial", "gpu", "d")


def _is_torch(a):
    try:
        import torch
    except ImportError:  # pragma: no cover
        return False
    return isinstance(a, torch.Tensor)


class nufft_3d:  # noqa: N801  (the reference's class name)
    """obj = nufft_3d(om, N, name, value, ...)"""

    def __init__(self, om, N=None, *varargin, device=None, tile=None, coils_per_pass=None,
                 samples_per_block=None, density_iters=20, verbose=False, tap_table=None, wait_polls=None,
                 spread_table=None, **kw):
        L = _lib.load()
        # name/value pairs (nufft_3d.m:71-76)
        if len(varargin) % 2:
            raise ValueError("'varargin' must be supplied in string/value pairs")
        pairs = dict(zip(varargin[0::2], varargin[1::2]))
        for k in pairs:
            if not isinstance(k, str):
                raise ValueError("'varargin' must be supplied in string/value pairs")
        pairs.update(kw)
        unknown = set(pairs) - set(_PROPS)
        if unknown:
            raise ValueError("unknown property %s" % sorted(unknown))
        om = np.asarray(om)
        if om.size == 0 or om.shape[0] != 3 or np.iscomplexobj(om) or not np.issubdtype(om.dtype, np.number):
            raise ValueError("om must be a real array with leading dimension of 3")
        om = np.ascontiguousarray(om.reshape(3, -1, order="F").T, dtype=np.float64)  # [3 x M] col-major
        self.M = om.shape[0]
        if N is None or np.size(N) == 0:
            N = 2 * np.ceil(np.max(np.abs(om), axis=0))
        Narr = np.asarray(N).reshape(-1)
        if Narr.size not in (1, 3):
            raise ValueError("N must be scalar or 3-vector of even integers")
        if np.any(Narr != np.round(Narr)):
            raise ValueError("N must be an even integer")
        Nc = (ctypes.c_int32 * 3)(*[int(v) for v in np.resize(Narr, 3)])
        opts = _lib.Opts()
        _lib.check(L.nufft3d_opts_default(ctypes.byref(opts)))
        if "J" in pairs:
            opts.J = float(pairs["J"])
        if "u" in pairs:
            opts.u = float(pairs["u"])
        if "alpha" in pairs:
            opts.alpha = float(pairs["alpha"])
        if "radial" in pairs:
            opts.radial = int(bool(pairs["radial"]))
        if "gpu" in pairs:
            opts.gpu = int(pairs["gpu"])
        if device is not None:
            opts.device = int(device)
        if tile is not None:
            for a in range(3):
                opts.tile[a] = int(tile[a])
        if coils_per_pass:
            opts.max_coils_per_pass = int(coils_per_pass)
        if samples_per_block:
            opts.max_samples_per_block = int(samples_per_block)
        opts.density_iters = int(density_iters) if density_iters > 0 else -1
        opts.verbose = int(bool(verbose))
        if tap_table is not None:  # True/1 build, False/0 on the fly, -1 auto (default)
            opts.tap_table = int(tap_table)
        if wait_polls is not None:  # polls of each bounded wait (0: give up at once)
            opts.wait_polls = int(wait_polls)
        if spread_table is not None:  # stored H' for the 8-coil spread: 1 build, 0 on the fly, -1 auto
            opts.spread_table = int(spread_table)
        dbuf = None
        if pairs.get("d") is not None:
            dbuf = np.ascontiguousarray(np.asarray(pairs["d"], dtype=np.float32).reshape(-1))
            if dbuf.size != self.M:
                raise ValueError("supplied density has wrong number of elements (should be %i)" % self.M)
            opts.d = dbuf.ctypes.data
        plan = ctypes.c_void_p()
        _lib.check(L.nufft3d_plan_create(om.ctypes.data, self.M, ctypes.cast(Nc, ctypes.c_void_p),
                                         int(Narr.size), ctypes.byref(opts), ctypes.byref(plan)))
        self._plan = plan
        self._L = L
        info = _lib.Info()
        _lib.check(L.nufft3d_plan_info(plan, ctypes.byref(info)))
        self._info = info
        self.N = np.array(info.N[:], dtype=np.int64)
        self.K = np.array(info.K[:], dtype=np.int64)
        self.nnz = int(info.nnz)
        self.J = info.J
        self.u = info.u
        self.alpha = info.alpha
        self.radial = bool(info.radial)
        self.gpu = 1
        self.tile = tuple(info.tile[:])
        self.n_blocks = int(info.n_blocks)
        self.taps_per_sample = info.taps_per_sample
        self.tap_table_bytes = int(info.tap_table_bytes)  # stored H (0: taps evaluated on the fly)
        self.spread_table_bytes = int(info.spread_table_bytes)  # stored H' (0: the spread evaluates the taps)
        self._adjoint = False
        if dbuf is not None and abs(float(np.mean(self.d)) - 1) > 1e-6:
            import warnings
            warnings.warn("mean(density) should be 1 (%f)" % float(np.mean(self.d)))

    # --------------------------------------------------------- lifecycle
    def close(self):
        if getattr(self, "_plan", None):
            if not getattr(self, "_borrowed", False):
                self._L.nufft3d_plan_destroy(self._plan)
            self._plan = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def share(self):
        """A second object on the same resident trajectory tables with its own
        work buffers and stream (nufft3d_plan_share); safe to use concurrently."""
        h = ctypes.c_void_p()
        _lib.check(self._L.nufft3d_plan_share(self.plan, ctypes.byref(h)))
        t = object.__new__(nufft_3d)
        t.__dict__.update(self.__dict__)
        t._plan = h
        t._adjoint = False
        return t

    def tune(self, nc, force=False):
        """Autotuner (nufft3d_plan_tune): times fNUFT+aNUFT of nc coils over
        piece sizes and coils per pass, keeps the fastest (cached per shape
        class).  Returns the choice and timings as a dict."""
        r = _lib.TuneResult()
        _lib.check(self._L.nufft3d_plan_tune(self.plan, int(nc), int(bool(force)), ctypes.byref(r)))
        self.n_blocks = int(self.info()["n_blocks"])
        return {"samples_per_block": r.samples_per_block, "coils_per_pass": r.coils_per_pass,
                "ms_best": r.ms_best, "ms_default": r.ms_default, "candidates": r.candidates,
                "from_cache": bool(r.from_cache)}

    def footprint(self, nc, with_solver=True):
        b = ctypes.c_int64()
        _lib.check(self._L.nufft3d_plan_footprint(self.plan, int(nc), int(bool(with_solver)), ctypes.byref(b)))
        return int(b.value)

    def check_status(self, stream=None):
        """Raises NufftError (NUFFT3D_ERR_TIMEOUT) if a bounded wait expired in
        device-pointer calls queued on `stream` (a torch.cuda.Stream, a raw
        handle, or None for torch's current stream) since the last check;
        synchronises that stream (nufft3d_check_status)."""
        if stream is None:
            import torch
            stream = torch.cuda.current_stream()
        h = getattr(stream, "cuda_stream", stream)
        _lib.check(self._L.nufft3d_check_status(self.plan, ctypes.c_void_p(h)))

    @property
    def plan(self):
        if not self._plan:
            raise RuntimeError("plan has been destroyed")
        return self._plan

    # -------------------------------------------------------- properties
    @property
    def U(self):
        out = np.empty(int(np.prod(self.N)), dtype=np.float32)
        _lib.check(self._L.nufft3d_get_deap(self.plan, out.ctypes.data))
        return out.reshape(tuple(self.N), order="F")

    @property
    def d(self):
        out = np.empty(self.M, dtype=np.float32)
        _lib.check(self._L.nufft3d_get_density(self.plan, out.ctypes.data))
        return out

    @property
    def nimg(self):
        return int(np.prod(self.N))

    def info(self):
        i = _lib.Info()
        _lib.check(self._L.nufft3d_plan_info(self.plan, ctypes.byref(i)))
        return {"N": list(i.N), "K": list(i.K), "M": i.M, "nnz": i.nnz, "tile": list(i.tile),
                "n_blocks": i.n_blocks, "taps_per_sample": i.taps_per_sample,
                "device_bytes": i.device_bytes, "tap_table_bytes": i.tap_table_bytes,
                "spread_table_bytes": i.spread_table_bytes}

    # --------------------------------------------------------- operators
    def _coils_img(self, x):
        n = x.numel() if _is_torch(x) else np.size(x)
        if n % self.nimg:
            raise ValueError("image size must be a multiple of prod(N) = %d" % self.nimg)
        return n // self.nimg

    def _coils_k(self, k):
        n = k.numel() if _is_torch(k) else np.size(k)
        if n % self.M:
            raise ValueError("data leading dimension(s) must be length %i" % self.M)
        return n // self.M

    @staticmethod
    def _stream_ptr(t):
        import torch
        return ctypes.c_void_p(torch.cuda.current_stream(t.device).cuda_stream)

    def fNUFT(self, x):  # noqa: N802
        """k = A*x (fNUFT.m): (N1,N2,N3[,nc]) -> (M, nc)."""
        if _is_torch(x):
            import torch
            nc = self._coils_img(x)
            x = x.contiguous()
            out = torch.empty((nc, self.M), dtype=torch.complex64, device=x.device)
            _lib.check(self._L.nufft3d_forward(self.plan, x.data_ptr(), out.data_ptr(), nc, self._stream_ptr(x)))
            return out
        nc = self._coils_img(x)
        xin = np.asfortranarray(np.asarray(x, dtype=np.complex64).reshape(tuple(self.N) + (nc,), order="F"))
        out = np.empty((self.M, nc), dtype=np.complex64, order="F")
        _lib.check(self._L.nufft3d_forward_host(self.plan, xin.ctypes.data, out.ctypes.data, nc))
        return out

    def aNUFT(self, k):  # noqa: N802
        """x = A'*k (aNUFT.m): (M[, nc]) -> (N1, N2, N3, nc)."""
        if _is_torch(k):
            import torch
            nc = self._coils_k(k)
            k = k.contiguous()
            out = torch.empty((nc,) + tuple(int(v) for v in self.N[::-1]), dtype=torch.complex64, device=k.device)
            _lib.check(self._L.nufft3d_adjoint(self.plan, k.data_ptr(), out.data_ptr(), nc, self._stream_ptr(k)))
            return out
        nc = self._coils_k(k)
        kin = np.asfortranarray(np.asarray(k, dtype=np.complex64).reshape(self.M, nc, order="F"))
        out = np.empty(tuple(self.N) + (nc,), dtype=np.complex64, order="F")
        _lib.check(self._L.nufft3d_adjoint_host(self.plan, kin.ctypes.data, out.ctypes.data, nc))
        return out

    def iprojection(self, x, damp=0.0, W=None):
        """y = A'(W.*(A x)) + damp^2 x (nufft_3d.m:305-313), device tensors only."""
        import torch
        nc = self._coils_img(x)
        x = x.contiguous()
        out = torch.empty_like(x)
        Wp = None
        if W is not None:
            W = W.contiguous().to(torch.float32)
            Wp = W.data_ptr()
        _lib.check(self._L.nufft3d_normal(self.plan, x.data_ptr(), out.data_ptr(), nc, float(damp), Wp,
                                          self._stream_ptr(x)))
        return out

    # mtimes / ctranspose: obj*x -> fNUFT, obj'*y -> aNUFT
    def ctranspose(self):
        t = object.__new__(nufft_3d)
        t.__dict__.update(self.__dict__)
        t._adjoint = not self._adjoint
        t._owner = self  # keep the plan alive
        t._plan = self._plan
        t._borrowed = True
        return t

    def mtimes(self, x):
        return self.aNUFT(x) if self._adjoint else self.fNUFT(x)

    def __mul__(self, x):
        return self.mtimes(x)

    def __matmul__(self, x):
        return self.mtimes(x)

    # ------------------------------------------------------------ solvers
    def _weights(self, W, nr, ny):
        """iNUFT.m:55-74 (the .*d is applied by the library)."""
        if W is None or np.isscalar(W) or np.size(W) <= 1:
            return None
        W = np.asarray(W, dtype=np.float64).reshape(-1)
        if W.size != self.M:
            if ny is None:
                ny = W.size
                nr = self.M / ny
            if nr % 1 or nr * ny != self.M:
                raise ValueError("W must be a vector of length ny or ny*nr")
            W = np.tile(W.reshape(1, ny), (int(nr), 1)).reshape(-1, order="F")
        if not np.all(np.isfinite(W)) or np.any(W < 0):
            raise ValueError("W must be finite and nonnegative")
        return np.ascontiguousarray(W, dtype=np.float32)

    def _raw_shape(self, raw):
        shape = tuple(raw.shape)
        nr = ny = None
        if shape[0] == self.M:
            nc = shape[1] if len(shape) > 1 else 1
            extra = int(np.prod(shape[2:])) if len(shape) > 2 else 1
        else:
            if len(shape) < 2 or shape[0] * shape[1] != self.M:
                raise ValueError("raw data leading dimension(s) must be length %i (not %s)" % (self.M, shape))
            nr, ny = shape[0], shape[1]
            nc = shape[2] if len(shape) > 2 else 1
            extra = int(np.prod(shape[3:])) if len(shape) > 3 else 1
        if extra > 1:
            raise ValueError("raw data size %s seems to have too many dimensions" % (shape,))
        return nc, nr, ny

    def iNUFT(self, raw, maxit=20, damp=0.0, W=None, constraint=None, lam=None, solver="minres",  # noqa: N802
              tol=1e-4, return_iters=False, x0=None):
        """im = obj.iNUFT(raw, maxit, damp, W) -> (N1, N2, N3, nc) (iNUFT.m).

        Each coil is solved as its own system; ``solver`` 'minres' (the
        reference's) or 'cg'; ``tol=0`` runs exactly ``maxit`` iterations.
        ``x0`` (same shape and kind as the result) starts the solve from an
        earlier image instead of zero, as discrep.m:55-58 does.
        """
        maxit = 20 if maxit is None else maxit
        phase = False
        if constraint:
            if constraint not in ("phase-constraint", "compressed-sensing", "parallel-imaging-sake",
                                  "parallel-imaging-pruno"):
                raise ValueError("unknown constraint")
            if constraint != "phase-constraint":
                raise NotImplementedError("constraint '%s' is not implemented (experimental in the reference, "
                                          "needs the external 'parallel' package)" % constraint)
            if lam is None:
                raise ValueError("lambda must be supplied with %s" % constraint)   # iNUFT.m:87-89
            if not (np.isscalar(lam) and np.isfinite(lam) and lam >= 0):
                raise ValueError("lambda must be a scalar finite nonnegative number")
            if x0 is not None:
                raise ValueError("x0 is not used with a constraint")
            phase = maxit > 1
            if not phase:
                import warnings
                warnings.warn("phase constraint is only effective when maxit>1")
        if not (np.isscalar(maxit) and np.isfinite(maxit) and maxit >= 0 and int(maxit) == maxit):
            raise ValueError("maxit must be a scalar nonnegative integer")
        damp = 0.0 if damp is None else damp
        if not (np.isscalar(damp) and np.isfinite(damp) and damp >= 0):
            raise ValueError("damp must be a scalar finite nonnegative number")
        sv = {"minres": _lib.SOLVER_MINRES, "cg": _lib.SOLVER_CG}[solver]
        if _is_torch(raw):
            import torch
            nc = self._coils_k(raw)
            raw = raw.contiguous()
            Wt = None
            if W is not None and not np.isscalar(W) and (W.numel() if _is_torch(W) else np.size(W)) > 1:
                Wn = W.detach().cpu().numpy() if _is_torch(W) else np.asarray(W)
                Wt = torch.from_numpy(self._weights(Wn, None, None)).to(raw.device)
            shape = (nc,) + tuple(int(v) for v in self.N[::-1])
            if x0 is not None:
                out = x0.detach().to(device=raw.device, dtype=torch.complex64).reshape(shape).contiguous().clone()
                fn = self._L.nufft3d_inverse_x0
            else:
                out = torch.empty(shape, dtype=torch.complex64, device=raw.device)
                fn = self._L.nufft3d_inverse
            its = (ctypes.c_int * nc)()
            wp = Wt.data_ptr() if Wt is not None else None
            if phase:
                _lib.check(self._L.nufft3d_inverse_phase(self.plan, raw.data_ptr(), out.data_ptr(), nc, int(maxit),
                                                         float(damp), float(lam), wp, float(tol),
                                                         ctypes.cast(its, ctypes.c_void_p), self._stream_ptr(raw)))
            else:
                _lib.check(fn(self.plan, raw.data_ptr(), out.data_ptr(), nc, int(maxit), float(damp), wp, sv,
                              float(tol), ctypes.cast(its, ctypes.c_void_p), self._stream_ptr(raw)))
            self.last_iters = list(its)
            return (out, list(its)) if return_iters else out
        raw = np.asarray(raw)
        nc, nr, ny = self._raw_shape(raw)
        if maxit <= 1 and W is not None and np.size(W) > 1:
            import warnings
            warnings.warn("weighting is only effective when maxit>1")
        Wf = self._weights(W, nr, ny)
        rin = np.asfortranarray(raw.astype(np.complex64).reshape(self.M, nc, order="F"))
        if x0 is not None:
            out = np.array(np.asarray(x0, dtype=np.complex64).reshape(tuple(self.N) + (nc,), order="F"),
                           dtype=np.complex64, order="F", copy=True)
            fn = self._L.nufft3d_inverse_x0_host
        else:
            out = np.empty(tuple(self.N) + (nc,), dtype=np.complex64, order="F")
            fn = self._L.nufft3d_inverse_host
        its = (ctypes.c_int * nc)()
        wp = Wf.ctypes.data if Wf is not None else None
        if phase:
            _lib.check(self._L.nufft3d_inverse_phase_host(self.plan, rin.ctypes.data, out.ctypes.data, nc,
                                                          int(maxit), float(damp), float(lam), wp, float(tol),
                                                          ctypes.cast(its, ctypes.c_void_p)))
        else:
            _lib.check(fn(self.plan, rin.ctypes.data, out.ctypes.data, nc, int(maxit), float(damp), wp, sv,
                          float(tol), ctypes.cast(its, ctypes.c_void_p)))
        self.last_iters = list(its)
        return (out, list(its)) if return_iters else out

    def discrep(self, data, stddev=None, iters=20, maxit=20, solver="minres"):
        """Discrepancy-principle estimate of damp (discrep.m:2-69).

        20 updates damp <- damp * discrepancy / |A x - data|, each solving
        (A'DA + damp^2 I) x = A'D data by MINRES (tol 1e-4, MATLAB's default
        maxit of 20) warm-started from the previous x, as discrep.m:50-66.
        """
        data = np.asarray(data)
        nc, _, _ = self._raw_shape(data)
        data = data.reshape(self.M, nc, order="F")
        if stddev is None:
            tmp = data[data != 0]
            tmp = np.concatenate([tmp.real, tmp.imag])
            stddev = float(np.median(np.abs(tmp - np.median(tmp))))
            import warnings
            warnings.warn("stddev not supplied. Guessing %.2e." % stddev)
        if not (np.isfinite(stddev) and stddev >= 0):
            raise ValueError("stddev must be a scalar finite nonnegative number")
        discrepancy = stddev * math.sqrt(data.size)
        damp = 0.1
        x = None
        for _ in range(iters):
            x = self.iNUFT(data, maxit, damp, None, solver=solver, tol=1e-4, x0=x)
            resnorm = float(np.linalg.norm(self.fNUFT(x) - data))
            damp = damp * (discrepancy / resnorm)
        return damp
