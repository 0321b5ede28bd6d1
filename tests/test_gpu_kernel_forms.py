"""GPU tests of the two device forms of the Kaiser-Bessel kernel and of the
iNUFT argument layouts.

* The device evaluates kernel.m's weights either as a polynomial fitted at
  plan time (Beatty alpha: max error < 4e-6 of the peak, checked at plan
  time) or, where that fit is not accurate enough (an explicit alpha = 25
  here), with the Numerical Recipes branches of kernel.m:14-30, whose
  large-argument branch uses a Cody-Waite exp onto ex2.approx.  Both are
  compared with the FP64 kernel.m of the oracle over the whole support:
  polynomial |dw| <= 4e-6; branches |dw| <= (1e-6 + 2.5e-7 |e|) w + 1e-12
  with e = alpha (sqrt(1 - d2/(J/2)^2) - 1) the exponent (FP32 rounding of
  the NR polynomials, rsqrt, and of e itself, which exp amplifies by |e|).
* fNUFT / aNUFT of a plan on the branch form against FP64 (rel L2 <= 1e-5).
* iNUFT with raw data in the [nr ny nc] layout and per-spoke weights W of
  length ny (iNUFT.m:27-38,55-74) against the oracle given the same layout
  and weights (rel L2 <= 1e-4).
"""
import ctypes

import numpy as np
import pytest

from nufft_3d_gb300 import _lib, nufft_3d, synth
from oracle.nufft_ref import NufftRef, kernel

pytestmark = pytest.mark.gpu
TOL_OP = 1e-5
TOL_IMG = 1e-4


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b)))


@pytest.mark.parametrize("alpha,poly", [(0.0, 1), (25.0, 0)])
def test_device_kernel_against_fp64(cuda, alpha, poly):
    torch = cuda
    J = 6.0
    om = synth.koosh_ball(16, 16, 200)
    obj = nufft_3d(om, 16, "J", J, "alpha", alpha, density_iters=0)
    info = _lib.Info()
    _lib.check(obj._L.nufft3d_plan_info(obj.plan, ctypes.byref(info)))
    assert info.kernel_polynomial == poly
    d2 = np.linspace(0.0, (J / 2) ** 2, 40001).astype(np.float32)
    d2_dev = torch.from_numpy(d2).cuda()
    w_dev = torch.empty_like(d2_dev)
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    _lib.check(obj._L.nufft3d_kernel_eval(obj.plan, d2_dev.data_ptr(), w_dev.data_ptr(), d2.size, s))
    w = w_dev.cpu().numpy().astype(np.float64)
    ref = kernel(d2.astype(np.float64), obj.alpha, J)
    err = np.abs(w - ref)
    print("alpha %g: max abs error %.2e, max relative error %.2e" % (obj.alpha, err.max(),
                                                                   float((err / np.maximum(ref, 1e-30)).max())))
    if poly:
        assert err.max() < 4e-6, err.max()
    else:
        # the large-argument branch is exp(e) * (...) with e = alpha (sqrt(t) - 1):
        # FP32 carries about |e| 2^-23 of absolute error in e, i.e. a relative
        # error of the weight that grows with |e| (the kernel's tail)
        e = np.abs(obj.alpha * (np.sqrt(1 - d2.astype(np.float64) / (J / 2) ** 2) - 1))
        bound = (1e-6 + 2.5e-7 * e) * ref + 1e-12
        assert np.all(err <= bound), float((err / bound).max())


def test_branch_form_operators_match_oracle(cuda):
    torch = cuda
    rng = np.random.default_rng(17)
    N, M, nc = 20, 4000, 2
    om = rng.uniform(-N / 2, N / 2 - 1, size=(3, M))
    obj = nufft_3d(om, N, "J", 6, "alpha", 25.0, density_iters=0)
    ref = NufftRef(om, N, J=6, alpha=25.0, density_iters=0)
    x = rng.standard_normal((N, N, N, nc)) + 1j * rng.standard_normal((N, N, N, nc))
    y = rng.standard_normal((M, nc)) + 1j * rng.standard_normal((M, nc))
    assert rel(obj.fNUFT(x), ref.fNUFT(x)) < TOL_OP
    assert rel(obj.aNUFT(y), ref.aNUFT(y)) < TOL_OP


@pytest.mark.parametrize("solver", ["minres", "cg"])
def test_readout_spoke_layout_and_per_spoke_weights(cuda, solver):
    rng = np.random.default_rng(18)
    N, nr, ny, nc = 24, 24, 300, 2
    om = synth.koosh_ball(N, nr, ny)       # readout r of spoke y at r + nr*y
    obj = nufft_3d(om, N, "J", 6)
    ref = NufftRef(om, N, J=6)
    raw = rng.standard_normal((nr, ny, nc)) + 1j * rng.standard_normal((nr, ny, nc))
    W = rng.uniform(0.5, 1.5, ny)          # one weight per spoke
    im = obj.iNUFT(raw, 6, 0.05, W, solver=solver, tol=0)
    imr = ref.iNUFT(raw, 6, 0.05, W, solver=solver, tol=0)
    assert im.shape == (N, N, N, nc)
    assert rel(im, imr) < TOL_IMG
    # the same data as [M nc] with the weights expanded per sample
    Wm = np.tile(W.reshape(1, ny), (nr, 1)).reshape(-1, order="F")
    im2 = obj.iNUFT(raw.reshape(nr * ny, nc, order="F"), 6, 0.05, Wm, solver=solver, tol=0)
    assert rel(im2, im) < 1e-6
    with pytest.raises(ValueError):
        obj.iNUFT(raw, 6, 0.05, W[:-1], solver=solver, tol=0)      # length neither ny nor nr*ny
