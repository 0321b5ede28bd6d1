"""GPU accuracy and status tests through the C ABI.

* Coils of very different gain in one interpolation pass: every coil of the
  adjoint (and the forward) within rel L2 1e-5 of the FP64 oracle, whatever
  the other coils of the pass hold (the spread's fixed-point scale is chosen
  per coil).
* The benchmark workload itself -- N=128^3, koosh ball 256 x 32768
  (M = 8,388,608), J=6, 8 coils of phantom x Gaussian coil maps -- fNUFT and
  aNUFT per coil against the FP64 matrix-free oracle (fNUFT.m:2-9,
  aNUFT.m:2-9), rel L2 <= 1e-5 each.
* An expired bounded wait in the gather is reported as NUFFT3D_ERR_TIMEOUT on
  the plan that ran it (device-pointer calls through nufft3d_check_status,
  host-pointer calls directly), and the context stays usable.
"""
import ctypes
import os

import numpy as np
import pytest

from nufft_3d_gb300 import _lib, nufft_3d, synth
from oracle.cpu_bench import adjoint_per_coil, forward_per_coil
from oracle.nufft_ref import NufftRef

pytestmark = pytest.mark.gpu
TOL_OP = 1e-5


def rel(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def img_to_dev(torch, x):
    return torch.from_numpy(np.ascontiguousarray(x.transpose(3, 2, 1, 0).astype(np.complex64))).cuda()


def img_from_dev(t):
    return t.cpu().numpy().transpose(3, 2, 1, 0)


def k_to_dev(torch, k):
    return torch.from_numpy(np.ascontiguousarray(np.asarray(k).T.astype(np.complex64))).cuda()


def k_from_dev(t):
    return t.cpu().numpy().T


GAINS = np.array([1.0, 1e-4, 3e2, 1e-2, 1.0, 5e-4, 1e1, 1e-3])


@pytest.mark.parametrize("nc", [8, 4, 3])
def test_coils_of_different_gain_in_one_pass(cuda, nc):
    """Coil gains spanning 3e2 .. 1e-4 in one pass: each coil <= 1e-5 against FP64."""
    torch = cuda
    rng = np.random.default_rng(21)
    N = 32
    om = synth.koosh_ball(N, 32, 1500)
    obj = nufft_3d(om, N, "J", 6, density_iters=0)
    ref = NufftRef(om, N, J=6, density_iters=0)
    g = GAINS[:nc]
    y = (rng.standard_normal((obj.M, nc)) + 1j * rng.standard_normal((obj.M, nc))) * g
    a = img_from_dev(obj.aNUFT(k_to_dev(torch, y)))
    ar = ref.aNUFT(y)
    errs = [rel(a[..., c], ar[..., c]) for c in range(nc)]
    assert max(errs) < TOL_OP, errs
    x = (rng.standard_normal((N, N, N, nc)) + 1j * rng.standard_normal((N, N, N, nc))) * g
    k = k_from_dev(obj.fNUFT(img_to_dev(torch, x)))
    kr = ref.fNUFT(x)
    errs = [rel(k[:, c], kr[:, c]) for c in range(nc)]
    assert max(errs) < TOL_OP, errs
    # a coil's result does not depend on the other coils of the pass (alone it
    # takes the fixed-point spread, about 22 bits per product; in a pass of 8
    # the stored H' in FP32 when the plan holds one)
    a1 = img_from_dev(obj.aNUFT(k_to_dev(torch, y[:, 1:2])))
    assert rel(a1[..., 0], a[..., 1]) < (5e-6 if obj.spread_table_bytes and nc >= 8 else 1e-6)


@pytest.mark.slow
def test_benchmark_workload_per_coil_parity(cuda):
    """N=128^3, koosh ball 256 x 32768, J=6, 8 coils (phantom x coil maps):
    fNUFT and aNUFT of every coil against the FP64 oracle, rel L2 <= 1e-5."""
    torch = cuda
    N, nr, ns, nc = 128, 256, 32768, 8
    om = synth.koosh_ball(N, nr, ns)
    im = synth.phantom_with_phase(N)[..., None] * synth.coil_maps(N, nc)
    obj = nufft_3d(om, N, "J", 6, "u", 2, density_iters=0)
    assert obj.M == nr * ns and obj.tap_table_bytes > 0  # the 8-coil gather reads the stored H
    ref = NufftRef(om, N, J=6, u=2, matrix=False, density_iters=0, workers=os.cpu_count())
    assert obj.nnz == ref.nnz
    k = k_from_dev(obj.fNUFT(img_to_dev(torch, im)))
    kr = forward_per_coil(ref, im)
    fwd = [rel(k[:, c], kr[:, c]) for c in range(nc)]
    # adjoint of the forward data plus complex noise at 30 dB SNR
    rng = np.random.default_rng(0)
    sig = np.sqrt(np.mean(np.abs(kr) ** 2, axis=0)) * 10 ** (-30 / 20)
    y = kr + sig * (rng.standard_normal(kr.shape) + 1j * rng.standard_normal(kr.shape)) / np.sqrt(2)
    del kr
    a = img_from_dev(obj.aNUFT(k_to_dev(torch, y)))
    ar = adjoint_per_coil(ref, y)
    adj = [rel(a[..., c], ar[..., c]) for c in range(nc)]
    print("per-coil rel L2 fwd", ["%.2e" % e for e in fwd], "adj", ["%.2e" % e for e in adj])
    assert max(fwd) < TOL_OP, fwd
    assert max(adj) < TOL_OP, adj


@pytest.mark.parametrize("nc", [2, 8])
def test_expired_wait_is_reported_on_its_plan(cuda, nc):
    """wait_polls=0: every bulk tile copy of the gather is still waited for
    before the block leaves, but counts as expired -- the timeout path runs
    without any fault.  Device-pointer calls report it through
    nufft3d_check_status (once; the flag is cleared), host-pointer calls
    directly; another plan on the device is unaffected."""
    torch = cuda
    N = 32  # K = 64: interior 8^3 tiles use the bulk tensor copy
    om = synth.koosh_ball(N, 32, 800)
    bad = nufft_3d(om, N, "J", 6, density_iters=0, wait_polls=0, tap_table=1)
    good = nufft_3d(om, N, "J", 6, density_iters=0, tap_table=1)
    L = _lib.load()
    stream = torch.cuda.current_stream()
    sp = ctypes.c_void_p(stream.cuda_stream)
    g = torch.Generator(device="cuda").manual_seed(1)
    x = torch.randn((nc, N, N, N), dtype=torch.complex64, device="cuda", generator=g)
    k = torch.empty((nc, bad.M), dtype=torch.complex64, device="cuda")
    kg = torch.empty_like(k)
    _lib.check(L.nufft3d_forward(bad.plan, x.data_ptr(), k.data_ptr(), nc, sp))
    _lib.check(L.nufft3d_forward(good.plan, x.data_ptr(), kg.data_ptr(), nc, sp))
    assert L.nufft3d_check_status(good.plan, sp) == _lib.SUCCESS
    assert L.nufft3d_check_status(bad.plan, sp) == _lib.ERR_TIMEOUT
    assert "did not complete" in _lib.last_error()
    assert L.nufft3d_check_status(bad.plan, sp) == _lib.SUCCESS  # read and cleared
    # the no-allocation forward reports on the same plan flag
    _lib.check(L.nufft3d_forward_noalloc(bad.plan, x.data_ptr(), k.data_ptr(), nc, sp))
    with pytest.raises(_lib.NufftError) as e:
        bad.check_status(stream)
    assert e.value.code == _lib.ERR_TIMEOUT
    # host-pointer entry points check the flag themselves
    xh = x.cpu().numpy().transpose(3, 2, 1, 0)
    with pytest.raises(_lib.NufftError) as e:
        bad.fNUFT(xh)
    assert e.value.code == _lib.ERR_TIMEOUT
    # the context is still usable: the good plan gives the oracle's answer
    ref = NufftRef(om, N, J=6, density_iters=0)
    assert rel(good.fNUFT(xh), ref.fNUFT(xh)) < TOL_OP
    assert rel(k_from_dev(kg), ref.fNUFT(xh)) < TOL_OP
    good.check_status(stream)
