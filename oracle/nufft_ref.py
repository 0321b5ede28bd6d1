"""FP64 CPU restatement of the marcsous/nufft_3d sparse-matrix path.

TEST INFRASTRUCTURE ONLY.  Only ``tests/``, ``__graft_entry__.smoke()`` and the
``cpu_baseline`` / ``--impl reference`` legs of ``bench.py`` may import this
module, and only as the checker (or as the timed CPU stand-in for the
reference).  The product path (``nufft_3d_gb300``) never calls it.

PARITY UNPINNED.  The reference is pure MATLAB; no MATLAB or Octave exists on
either machine and the reference ships no golden vectors or known-answer
tests.  This restatement is therefore checked against independent known
answers instead (A&S/NR bounds of I0 against ``scipy.special.i0``, the
closed-form Beatty alpha, the analytic Lewitt deapodization that the reference
keeps disabled in ``deap.m:38-95``, the Cartesian full-grid case of
``test_nufft3d.m:46-52`` against a plain FFT, the exact adjoint identity and
diag(Q'Q) ~ 1 from ``density.m:44-82``), see ``tests/test_oracle.py``.

Conventions follow the reference file by file (paths relative to the
reference project root):

* ``@nufft_3d/nufft_3d.m:79-111``   argument checks, Beatty alpha, K.
* ``@nufft_3d/nufft_3d.m:119-126``  om scaling and the in-bounds mask ``ok``.
* ``@nufft_3d/nufft_3d.m:153-212``  neighbour set, weights (rounded to single,
  ``:160``), column-major grid index with mod-K wrap.
* ``@nufft_3d/kernel.m:2-34``       Kaiser-Bessel kernel with the Numerical
  Recipes / Abramowitz-Stegun 9.8.1-9.8.2 polynomial, complex branch, x2 hack.
* ``@nufft_3d/deap.m:2-36,97-98``   deapodization from untruncated kernel
  samples via length-2K symmetric inverse FFTs.
* ``@nufft_3d/density.m:2-42``      Pipe-style density iteration.
* ``@nufft_3d/nufft_3d.m:285-302``  fft3_pad / ifft3_crop.
* ``@nufft_3d/fNUFT.m``, ``@nufft_3d/aNUFT.m``  operators with 1/sqrt(nnz).
* ``@nufft_3d/nufft_3d.m:305-313``  iprojection (normal operator).
* ``@nufft_3d/iNUFT.m:25-138``      iNUFT default path (W = d, MINRES tol 1e-4).

Array conventions: images are numpy arrays of shape (N1, N2, N3[, nc]) read
in MATLAB column-major order (``order='F'``); sample data is (M, nc).
"""
from __future__ import annotations

import math
import numpy as np
import scipy.sparse as sp

# Numerical Recipes bessi0 coefficients (Abramowitz & Stegun 9.8.1 / 9.8.2),
# as used by kernel.m:22-30.
_NR_SMALL = (1.0, 3.5156229, 3.0899424, 1.2067492, 0.2659732, 0.360768e-1,
             0.45813e-2)
_NR_LARGE = (0.39894228, 0.1328592e-1, 0.225319e-2, -0.157565e-2,
             0.916281e-2, -0.2057706e-1, 0.2635537e-1, -0.1647633e-1,
             0.392377e-2)


def _horner(y, coeffs):
    acc = coeffs[-1] * np.ones_like(y)
    for c in reversed(coeffs[:-1]):
        acc = c + y * acc
    return acc


def bessi0(ax):
    """I0 as kernel.m:14-34 computes it (real or complex argument)."""
    ax = np.asarray(ax)
    out = np.zeros(ax.shape, dtype=ax.dtype)
    k = np.abs(ax) < 3.75
    y = ax[k] / 3.75
    y = y * y
    out[k] = _horner(y, _NR_SMALL)
    kl = ~k
    a = ax[kl]
    y = 3.75 / a
    out[kl] = (np.exp(a) / np.sqrt(a)) * _horner(y, _NR_LARGE)
    # kernel.m:32-34: "hack to get the same result as MATLAB besseli"
    hack = kl & (np.real(ax) == 0)
    out[hack] = 2 * out[hack]
    return out


def kernel(dist2, alpha, J):
    """Kaiser-Bessel kernel of kernel.m:2-11 for an array of squared distances.

    Elements with dist2 > (J/2)^2 take MATLAB's complex sqrt branch
    (0 + i*sqrt(|t|)), everything else stays real, exactly as the element-wise
    MATLAB evaluation of a real scalar/array would.
    """
    dist2 = np.atleast_1d(np.asarray(dist2, dtype=np.float64))
    t = 1 - dist2 / (J / 2) ** 2
    out = np.empty(dist2.shape, dtype=np.float64)
    den = bessi0(np.array([alpha], dtype=np.float64))[0]
    pos = t >= 0
    if pos.any():
        arg = alpha * np.sqrt(t[pos])
        out[pos] = np.real(bessi0(arg) / den)
    if (~pos).any():
        arg = (alpha * (0.0 + 1j * np.sqrt(-t[~pos]))).astype(np.complex128)
        out[~pos] = np.real(bessi0(arg) / den)
    return out


def beatty_alpha(J, u, radial):
    """nufft_3d.m:85-92."""
    if radial:
        return math.pi * math.sqrt(J ** 2 * (1 - 0.5 / u) ** 2 - 0.6 * u)
    return math.pi * math.sqrt(J ** 2 * (1 - 0.5 / u) ** 2 - 0.8)


class NufftRef:
    """FP64 restatement of the ``@nufft_3d`` object (sparse-matrix form).

    ``om`` is [3, M] in cycles/FOV, ``N`` a scalar or 3-vector (even).
    ``matrix`` selects the literal scipy CSR build (default) or lazy use of
    the matrix-free C restatement in ``oracle/interp_ref.c`` for large M.
    """

    def __init__(self, om, N, J=4, u=2, alpha=0, radial=True, d=None,
                 matrix=True, density_iters=20, workers=None):
        self.workers = workers  # scipy.fft threads (None: numpy.fft)
        om = np.asarray(om)
        if om.ndim < 1 or om.shape[0] != 3 or om.size == 0 or np.iscomplexobj(om):
            raise ValueError("om must be a real array with leading dimension of 3")
        om = om.reshape(3, -1)
        self.J = float(J)
        self.u = float(u)
        self.radial = bool(radial)
        if self.u < 1 or self.u > 6:
            raise ValueError("value of u=%f is not recommended" % self.u)
        if alpha == 0:
            alpha = beatty_alpha(self.J, self.u, self.radial)
        self.alpha = float(alpha)
        Nv = np.ones(3) * np.asarray(N, dtype=np.float64).reshape(-1)
        if np.asarray(N).size not in (1, 3):
            raise ValueError("N must be scalar or 3-vector of even integers")
        if np.all(Nv == 0) or Nv[0] % 2 or Nv[1] % 2:
            raise ValueError("N must be an even integer")
        if np.all(om[2] == 0):
            Nv[2] = 1
        self.N = Nv.astype(np.int64)
        K = 2 * np.ceil(Nv * self.u / 2)
        if self.N[2] == 1:
            K[2] = 1
        if np.prod(K) >= 2 ** 31 - 1:
            raise ValueError("N or u too large")
        self.K = K.astype(np.int64)
        self.om_g = self.u * om.astype(np.float64)      # nufft_3d.m:120
        K = self.K
        ok = (self.om_g[0] >= -K[0] / 2) & (self.om_g[0] <= K[0] / 2 - 1)
        ok = (self.om_g[1] >= -K[1] / 2) & (self.om_g[1] <= K[1] / 2 - 1) & ok
        # nufft_3d.m:125 -- '&' binds tighter than '|': in 2D every point is kept
        ok = ((self.om_g[2] >= -K[2] / 2) & (self.om_g[2] <= K[2] / 2 - 1) & ok) | (self.N[2] == 1)
        self.ok = ok
        self.nnz = int(ok.sum())
        self.M = om.shape[1]
        self.H = self._build_H() if matrix else None
        self.U = self.deap()
        if d is None:
            self.d = self.density(density_iters)
        else:
            d = np.asarray(d, dtype=np.float64).reshape(-1).copy()
            if d.size != self.M:
                raise ValueError("supplied density has wrong number of elements (should be %i)" % self.M)
            d[~ok] = 0
            self.d = d

    # ------------------------------------------------------------------ setup
    def offsets(self):
        R = math.ceil(self.J / 2)
        return range(-R, R + 1)

    def _build_H(self):
        """nufft_3d.m:153-212: COO triplets per offset, weights rounded to single."""
        rows, cols, vals = [], [], []
        K = self.K
        og = self.om_g
        rx, ry, rz = np.round(og[0]), np.round(og[1]), np.round(og[2])
        rx = np.where(np.abs(og[0] - np.trunc(og[0])) == 0.5, np.trunc(og[0]) + np.sign(og[0]), rx)
        ry = np.where(np.abs(og[1] - np.trunc(og[1])) == 0.5, np.trunc(og[1]) + np.sign(og[1]), ry)
        rz = np.where(np.abs(og[2] - np.trunc(og[2])) == 0.5, np.trunc(og[2]) + np.sign(og[2]), rz)
        idx_all = np.arange(self.M)
        J2 = self.J ** 2
        for dx in self.offsets():
            for dy in self.offsets():
                for dz in self.offsets():
                    if self.N[2] == 1 and dz != 0:
                        continue
                    x = rx + dx
                    y = ry + dy
                    z = rz + dz
                    dx2 = (x - og[0]) ** 2
                    dy2 = (y - og[1]) ** 2
                    dz2 = (z - og[2]) ** 2
                    x = np.mod(x, K[0])
                    y = np.mod(y, K[1])
                    z = np.mod(z, K[2])
                    if self.radial:
                        dist2 = dx2 + dy2 + dz2
                        i = self.ok & (4 * dist2 <= J2)
                        s = kernel(dist2[i], self.alpha, self.J)
                    else:
                        i = self.ok & (4 * dx2 <= J2) & (4 * dy2 <= J2) & (4 * dz2 <= J2)
                        s = (kernel(dx2[i], self.alpha, self.J) * kernel(dy2[i], self.alpha, self.J)
                             * kernel(dz2[i], self.alpha, self.J))
                    j = x[i] + K[0] * y[i] + K[0] * K[1] * z[i]
                    rows.append(idx_all[i])
                    cols.append(j.astype(np.int64))
                    vals.append(s.astype(np.float32).astype(np.float64))
        rows = np.concatenate(rows)
        cols = np.concatenate(cols)
        vals = np.concatenate(vals)
        return sp.csr_matrix((vals, (rows, cols)), shape=(self.M, int(np.prod(K))))

    def deap(self):
        """deap.m:2-36 and :97-98 (numerical, untruncated kernel)."""
        J = int(math.floor(self.J))
        nz = 1 if self.N[2] == 1 else J + 1
        T = np.zeros((J + 1, J + 1, nz))
        for dx in range(J + 1):
            for dy in range(J + 1):
                for dz in range(nz):
                    dx2, dy2, dz2 = (dx / 2) ** 2, (dy / 2) ** 2, (dz / 2) ** 2
                    if self.radial:
                        T[dx, dy, dz] = kernel(dx2 + dy2 + dz2, self.alpha, self.J)[0]
                    else:
                        T[dx, dy, dz] = (kernel(dx2, self.alpha, self.J)[0] * kernel(dy2, self.alpha, self.J)[0]
                                         * kernel(dz2, self.alpha, self.J)[0])
        U = T
        ndim = 2 if nz == 1 else 3
        for j in range(ndim):
            Kj = int(self.K[j])
            Nj = int(self.N[j])
            # ifft(U*K, 2K, j, 'symmetric') == irfft of the first K+1 entries
            Uz = np.moveaxis(U * Kj, j, 0)
            full = np.zeros((Kj + 1,) + Uz.shape[1:])
            n = min(Uz.shape[0], Kj + 1)
            full[:n] = Uz[:n]
            out = np.fft.irfft(full, n=2 * Kj, axis=0)
            keep = np.concatenate([out[:Nj // 2], out[2 * Kj - Nj // 2:]], axis=0)
            U = np.moveaxis(keep, 0, j)
        U = np.fft.fftshift(U)
        if U.ndim == 2:
            U = U[:, :, None]
        return 1.0 / U

    def density(self, maxit=20):
        """density.m:2-14,42 in float64 (the reference's gpu=0 class)."""
        d = self.ok.astype(np.float64)
        eps = np.finfo(np.float64).eps
        for _ in range(maxit):
            HHd = self.spmv(self.spmv_t(d))
            d = d / np.maximum(HHd, eps)
        return d / (d.sum() / self.nnz)

    # ----------------------------------------------------------- primitives
    def spmv(self, k):
        """nufft_3d.m:259-271: H * k (complex or real)."""
        if self.H is not None:
            return self.H @ k
        from oracle.interp_ref import interp_forward
        return interp_forward(self, k)

    def spmv_t(self, k):
        """nufft_3d.m:274-282: H' * k."""
        if self.H is not None:
            return self.H.T @ k
        from oracle.interp_ref import interp_adjoint
        return interp_adjoint(self, k)

    def fft3_pad(self, x):
        """nufft_3d.m:285-291 (x has shape (N1,N2,N3,nc))."""
        for j in range(3):
            pad = (int(self.K[j]) - int(self.N[j])) // 2
            widths = [(0, 0)] * x.ndim
            widths[j] = (pad, pad)
            x = np.pad(x, widths)
            x = self._fft(np.fft.fftshift(x, axes=j), j, inverse=False)
        return x

    def _fft(self, x, axis, inverse):
        if self.workers:
            import scipy.fft as sf
            return (sf.ifft if inverse else sf.fft)(x, axis=axis, workers=self.workers)
        return (np.fft.ifft if inverse else np.fft.fft)(x, axis=axis)

    def ifft3_crop(self, k):
        """nufft_3d.m:294-302."""
        for j in range(3):
            mid = (int(self.K[j]) - int(self.N[j])) // 2
            k = np.fft.ifftshift(self._fft(k, j, inverse=True), axes=j) * self.K[j]
            sl = [slice(None)] * k.ndim
            sl[j] = slice(mid, int(self.K[j]) - mid)
            k = k[tuple(sl)]
        return k

    # ------------------------------------------------------------ operators
    def fNUFT(self, x):
        """fNUFT.m:2-9 -> (M, nc) complex."""
        N = self.N
        k = np.asarray(x, dtype=np.complex128).reshape(N[0], N[1], N[2], -1, order="F")
        k = k * self.U[..., None]
        k = self.fft3_pad(k)
        k = k.reshape(int(np.prod(self.K)), -1, order="F")
        k = self.spmv(k)
        return k / math.sqrt(self.nnz)

    def aNUFT(self, k):
        """aNUFT.m:2-9 -> (N1, N2, N3, nc) complex."""
        x = np.asarray(k, dtype=np.complex128).reshape(self.M, -1, order="F")
        x = self.spmv_t(x)
        K = self.K
        x = x.reshape(K[0], K[1], K[2], -1, order="F")
        x = self.ifft3_crop(x)
        x = x * self.U[..., None]
        return x / math.sqrt(self.nnz)

    def iprojection(self, x, damp, W):
        """nufft_3d.m:305-313 (no nullspace branch): (prod(N), nc)."""
        y = self.fNUFT(x)
        y = np.asarray(W).reshape(-1, 1) * y if np.ndim(W) else W * y
        y = self.aNUFT(y)
        x = np.asarray(x).reshape(y.shape, order="F")
        y = y + damp ** 2 * x
        return y.reshape(int(np.prod(self.N)), -1, order="F")

    def weights(self, W=None, nr=None, ny=None):
        """iNUFT.m:55-74: W default = d; per-spoke (ny) or per-sample weights."""
        if W is None or np.isscalar(W) or np.size(W) <= 1:
            return self.d
        W = np.asarray(W, dtype=np.float64)
        nrow = self.M
        if W.size != nrow:
            if ny is None:
                ny = W.size
                nr = nrow / ny
            if nr % 1 or nr * ny != nrow:
                raise ValueError("W must be a vector of length ny or ny*nr")
            W = np.tile(W.reshape(1, ny), (int(nr), 1))
        W = W.reshape(nrow, order="F") * self.d
        if not np.all(np.isfinite(W)) or np.any(W < 0):
            raise ValueError("W must be finite and nonnegative")
        return W

    def iNUFT_phase(self, raw, maxit, damp, lam, W=None, tol=1e-4):
        """iNUFT.m:140-168 'phase-constraint' with pprojection (nufft_3d.m:325-334).

        x from the plain MINRES solve; P = exp(i angle(convn(x, ones(3),
        'same'))) -- ones(3) is 3x3, so the box runs over x-y per slice with
        zero padding; then (P'A'WAP + damp^2 + i lam^2 imag) y = P'A'W raw by
        CG with real inner products from y = 0 (the reference's pcgpc is
        external); returns P y."""
        x = self.iNUFT(raw, maxit, damp, W, solver="minres", tol=tol)
        if maxit <= 1:
            return x
        N = self.N
        nc = x.shape[3]
        raw = np.asarray(raw, dtype=np.complex128).reshape(self.M, nc, order="F")
        Wv = self.weights(W, None, None)
        P = np.zeros_like(x)
        pad = np.pad(x, ((1, 1), (1, 1), (0, 0), (0, 0)))
        for dx in range(3):
            for dy in range(3):
                P += pad[dx:dx + N[0], dy:dy + N[1]]
        P = np.exp(1j * np.angle(P))
        b = np.conj(P) * self.aNUFT(Wv[:, None] * raw)
        n = int(np.prod(N))
        out = np.zeros((n, nc), dtype=np.complex128)
        self.last_iters = []
        for c in range(nc):
            Pc = P[..., c].reshape(n, order="F")

            def A(y, Pc=Pc):
                t = self.iprojection(Pc * y, damp, Wv)[:, 0]
                return np.conj(Pc) * t + 1j * lam ** 2 * y.imag
            y, it = cg(A, b[..., c].reshape(n, order="F"), tol, maxit)
            self.last_iters.append(it)
            out[:, c] = Pc * y
        return out.reshape(N[0], N[1], N[2], nc, order="F")

    def iNUFT(self, raw, maxit=20, damp=0.0, W=None, solver="minres", tol=1e-4, x0=None):
        """iNUFT.m:25-138 default path; per-coil systems; returns (N1,N2,N3,nc).

        x0 (N1,N2,N3,nc) starts each solve from an earlier image, as the
        minres(..., x) call of discrep.m:58 does."""
        raw = np.asarray(raw, dtype=np.complex128)
        nr = ny = None
        if raw.shape[0] == self.M:
            nc = raw.shape[1] if raw.ndim > 1 else 1
        else:
            nr, ny = raw.shape[0], raw.shape[1]
            if nr * ny != self.M:
                raise ValueError("raw data leading dimension(s) must be length %i" % self.M)
            nc = raw.shape[2] if raw.ndim > 2 else 1
        raw = raw.reshape(self.M, nc, -1, order="F")
        if raw.shape[2] > 1:
            raise ValueError("raw data size seems to have too many dimensions")
        raw = raw[:, :, 0]
        Wv = self.weights(W, nr, ny)
        N = self.N
        if maxit == 0:
            return self.aNUFT(Wv[:, None] * raw)
        b = self.aNUFT(Wv[:, None] * raw).reshape(int(np.prod(N)), nc, order="F")
        out = np.zeros_like(b)
        X0 = None if x0 is None else np.asarray(x0, dtype=np.complex128).reshape(int(np.prod(N)), nc, order="F")
        self.last_iters = []
        for c in range(nc):
            A = lambda v: self.iprojection(v, damp, Wv)[:, 0]
            xc = None if X0 is None else X0[:, c]
            if solver == "minres":
                x, it = minres(A, b[:, c], tol, maxit, xc)
            else:
                x, it = cg(A, b[:, c], tol, maxit, xc)
            self.last_iters.append(it)
            out[:, c] = x
        return out.reshape(N[0], N[1], N[2], nc, order="F")

    # ------------------------------------------------------------- checks
    def nudft(self, x):
        """Direct NUDFT of the implied continuous transform (small N only).

        fNUFT(x)[m] ~ c * sum_n x[n] exp(-2 pi i om_m . (n - N/2) / N).
        """
        N = self.N
        x = np.asarray(x, dtype=np.complex128).reshape(N[0], N[1], N[2], -1, order="F")
        om = self.om_g / self.u
        out = np.zeros((self.M, x.shape[3]), dtype=np.complex128)
        grids = [np.arange(int(N[a])) - int(N[a]) // 2 for a in range(3)]
        ex = np.exp(-2j * np.pi * np.outer(om[0], grids[0]) / N[0])
        ey = np.exp(-2j * np.pi * np.outer(om[1], grids[1]) / N[1])
        ez = np.exp(-2j * np.pi * np.outer(om[2], grids[2]) / max(N[2], 1))
        for c in range(x.shape[3]):
            t = np.einsum("mz,xyz->mxy", ez, x[..., c])
            t = np.einsum("my,mxy->mx", ey, t)
            out[:, c] = np.einsum("mx,mx->m", ex, t)
        out[~self.ok] = 0
        return out


def discrep(ref, data, stddev, iters=20, maxit=20, solver="minres"):
    """discrep.m:2-69: damp <- damp * discrepancy/|A x - data|, 20 times, x
    from MINRES (tol 1e-4, maxit 20) warm-started from the previous x."""
    data = np.asarray(data, dtype=np.complex128).reshape(ref.M, -1, order="F")
    discrepancy = stddev * math.sqrt(data.size)
    damp, x = 0.1, None
    for _ in range(iters):
        x = ref.iNUFT(data, maxit, damp, None, solver=solver, tol=1e-4, x0=x)
        resnorm = float(np.linalg.norm(ref.fNUFT(x) - data))
        damp = damp * (discrepancy / resnorm)
    return damp


def cg(A, b, tol, maxit, x0=None):
    """Conjugate gradients with FP64 scalars from x0 (default 0); stop when
    |r| <= tol*|b| (tol=0: fixed count)."""
    x = np.zeros_like(b) if x0 is None else np.array(x0, dtype=b.dtype)
    r = b.copy() if x0 is None else b - A(x)
    p = r.copy()
    rr = np.vdot(r, r).real
    nb = math.sqrt(np.vdot(b, b).real)
    it = 0
    for it in range(1, maxit + 1):
        q = A(p)
        alpha = rr / np.vdot(p, q).real
        x = x + alpha * p
        r = r - alpha * q
        rr_new = np.vdot(r, r).real
        if tol > 0 and math.sqrt(rr_new) <= tol * nb:
            break
        p = r + (rr_new / rr) * p
        rr = rr_new
    return x, it


def minres(A, b, tol, maxit, x0=None):
    """MINRES (Paige & Saunders 1975) for Hermitian A from x0 (default 0), no
    preconditioner; with x0 the recurrence runs on r0 = b - A x0 and x0 is
    added to its iterate (MATLAB minres with x0).

    Lanczos order: p = A v - beta v_prev; alpha = <v, p>; p -= alpha v.
    Stops when the recurrence's residual estimate satisfies ||r||/||b|| <= tol
    (the relres test of iNUFT.m:114,136); tol=0 forces exactly ``maxit`` steps.
    Scalars are FP64.
    """
    x = np.zeros_like(b) if x0 is None else np.array(x0, dtype=b.dtype)
    r0 = b if x0 is None else b - A(x)
    nb = math.sqrt(np.vdot(b, b).real)
    beta1 = math.sqrt(np.vdot(r0, r0).real)
    if beta1 == 0:
        return x, 0
    v_prev = np.zeros_like(b)
    v = r0 / beta1
    beta = beta1
    w1 = np.zeros_like(b)
    w2 = np.zeros_like(b)
    dbar = 0.0
    epsln = 0.0
    phibar = beta1
    cs, sn = -1.0, 0.0
    it = 0
    for it in range(1, maxit + 1):
        p = A(v)
        p = p - beta * v_prev
        alpha = np.vdot(v, p).real
        p = p - alpha * v
        beta_next = math.sqrt(np.vdot(p, p).real)
        oldeps = epsln
        delta = cs * dbar + sn * alpha
        gbar = sn * dbar - cs * alpha
        epsln = sn * beta_next
        dbar = -cs * beta_next
        gamma = max(math.hypot(gbar, beta_next), np.finfo(np.float64).eps)
        cs = gbar / gamma
        sn = beta_next / gamma
        phi = cs * phibar
        phibar = sn * phibar
        w = (v - oldeps * w1 - delta * w2) / gamma
        x = x + phi * w
        w1, w2 = w2, w
        v_prev = v
        if beta_next > 0:
            v = p / beta_next
        beta = beta_next
        if tol > 0 and phibar <= tol * nb:
            break
        if beta_next == 0:
            break
    return x, it
