"""GPU parity: libnufft3d (through the C ABI) against the FP64 oracle.

Tolerances: forward/adjoint relative L2 <= 1e-5 and iterative images <= 1e-4
against FP64 (the accuracy targets of the port); the sm_103a kernels compute
in FP32 with FP64 solver scalars.
"""
import glob
import math
import os

import numpy as np
import pytest

from nufft_3d_gb300 import nufft_3d, synth
from oracle.nufft_ref import NufftRef

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
TOL_OP = 1e-5
TOL_IMG = 1e-4


def rel(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def img_to_dev(torch, x):
    """(N1,N2,N3,nc) column-major numpy -> (nc,N3,N2,N1) contiguous cuda tensor."""
    x = x.reshape(x.shape[:3] + (-1,), order="F") if x.ndim == 3 else x
    return torch.from_numpy(np.ascontiguousarray(x.transpose(3, 2, 1, 0).astype(np.complex64))).cuda()


def img_from_dev(t):
    return t.cpu().numpy().transpose(3, 2, 1, 0)


def k_to_dev(torch, k):
    return torch.from_numpy(np.ascontiguousarray(np.asarray(k).reshape(k.shape[0], -1).T.astype(np.complex64))).cuda()


def k_from_dev(t):
    return t.cpu().numpy().T


@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(GOLDEN, "*.npz"))))
def test_golden(cuda, path):
    torch = cuda
    z = np.load(path)
    obj = nufft_3d(z["om"], int(z["N"]), "J", float(z["J"]), "u", float(z["u"]), "radial", int(z["radial"]))
    assert obj.nnz == int(z["nnz"])
    assert obj.alpha == pytest.approx(float(z["alpha"]), rel=1e-15)
    np.testing.assert_allclose(obj.U, z["U"], rtol=1e-6)
    assert rel(obj.d, z["d"]) < 1e-4
    k = k_from_dev(obj.fNUFT(img_to_dev(torch, z["x"])))
    assert rel(k, z["k"]) < TOL_OP
    a = img_from_dev(obj.aNUFT(k_to_dev(torch, z["y"])))
    assert rel(a, z["a"]) < TOL_OP
    # host-pointer variants give the same numbers
    kh = obj.fNUFT(z["x"])
    assert rel(kh, k) < 1e-6
    ah = obj.aNUFT(z["y"])
    assert rel(ah, a) < 1e-6
    damp, maxit = float(z["damp"]), int(z["maxit"])
    assert rel(obj.iNUFT(z["raw"], 0), z["im_regrid"]) < TOL_OP
    im = obj.iNUFT(z["raw"], maxit, damp, solver="minres", tol=0)
    assert rel(im, z["im_minres"]) < TOL_IMG
    im = obj.iNUFT(z["raw"], maxit, damp, solver="cg", tol=0)
    assert rel(im, z["im_cg"]) < TOL_IMG


@pytest.mark.parametrize("opts,nc", [
    (dict(J=6, u=2, radial=1), 1),
    (dict(J=6, u=2, radial=1), 3),
    (dict(J=6, u=2, radial=1), 12),
    (dict(J=4, u=2, radial=0), 2),
    (dict(J=7, u=1.5, radial=1), 1),
    (dict(J=2, u=2, radial=1), 1),
])
def test_random_trajectory_parity(cuda, opts, nc):
    torch = cuda
    rng = np.random.default_rng(7)
    N, M = 20, 4000
    om = rng.uniform(-N / 2 - 1, N / 2, size=(3, M))  # some samples out of bounds
    obj = nufft_3d(om, N, *sum(([k, v] for k, v in opts.items()), []), density_iters=0)
    ref = NufftRef(om, N, density_iters=0, **opts)
    assert obj.nnz == ref.nnz and obj.nnz < M
    x = rng.standard_normal((N, N, N, nc)) + 1j * rng.standard_normal((N, N, N, nc))
    y = rng.standard_normal((M, nc)) + 1j * rng.standard_normal((M, nc))
    k = k_from_dev(obj.fNUFT(img_to_dev(torch, x)))
    kr = ref.fNUFT(x)
    assert rel(k, kr) < TOL_OP
    assert np.all(k[~ref.ok] == 0)
    a = img_from_dev(obj.aNUFT(k_to_dev(torch, y)))
    assert rel(a, ref.aNUFT(y)) < TOL_OP


def test_phantom_N64_plain_method(cuda):
    """N=64 phantom with phase, 64 x 4096 golden-angle koosh ball, J=6, 1 coil:
    fNUFT, aNUFT and 20-iteration CG with damp 1e-3 against the FP64 oracle."""
    torch = cuda
    N = 64
    om = synth.koosh_ball(N, 64, 4096)
    obj = nufft_3d(om, N, "J", 6, "u", 2)
    ref = NufftRef(om, N, J=6, u=2, matrix=False)
    assert obj.nnz == ref.nnz == om.shape[1]
    assert rel(obj.d, ref.d) < 1e-4
    x = synth.phantom_with_phase(N)
    k = k_from_dev(obj.fNUFT(img_to_dev(torch, x)))
    kr = ref.fNUFT(x)
    assert rel(k, kr) < TOL_OP
    a = img_from_dev(obj.aNUFT(k_to_dev(torch, kr)))
    assert rel(a, ref.aNUFT(kr)) < TOL_OP
    im = obj.iNUFT(kr, 20, 1e-3, solver="cg", tol=0)
    imr = ref.iNUFT(kr, 20, 1e-3, solver="cg", tol=0)
    assert rel(im, imr) < TOL_IMG


def test_normal_operator_matches_composition(cuda):
    torch = cuda
    rng = np.random.default_rng(3)
    N, M, nc = 24, 6000, 2
    om = rng.uniform(-N / 2, N / 2 - 1, size=(3, M))
    obj = nufft_3d(om, N, "J", 6)
    x = img_to_dev(torch, rng.standard_normal((N, N, N, nc)) + 1j * rng.standard_normal((N, N, N, nc)))
    damp = 0.3
    y = obj.iprojection(x, damp)
    d = torch.from_numpy(obj.d).cuda()
    k = obj.fNUFT(x) * d[None, :]
    y2 = obj.aNUFT(k) + damp ** 2 * x
    assert float((y - y2).abs().norm() / y2.abs().norm()) < 1e-5


def test_adjoint_identity_large(cuda):
    torch = cuda
    N = 96
    om = synth.koosh_ball(N, 96, 6000)
    obj = nufft_3d(om, N, "J", 6, density_iters=0)
    g = torch.Generator(device="cuda").manual_seed(0)
    nc = 2
    x = torch.randn((nc, N, N, N), dtype=torch.complex64, device="cuda", generator=g)
    y = torch.randn((nc, obj.M), dtype=torch.complex64, device="cuda", generator=g)
    lhs = torch.vdot(y.flatten().to(torch.complex128), obj.fNUFT(x).flatten().to(torch.complex128))
    rhs = torch.vdot(obj.aNUFT(y).flatten().to(torch.complex128), x.flatten().to(torch.complex128))
    assert abs(complex(lhs - rhs)) / abs(complex(lhs)) < 1e-5


def test_two_d_mode(cuda):
    rng = np.random.default_rng(4)
    N, M = 32, 3000
    om = np.vstack([rng.uniform(-20, 20, (2, M)), np.zeros((1, M))])  # some beyond the grid: 2D keeps all
    obj = nufft_3d(om, N, "J", 4, density_iters=0)
    ref = NufftRef(om, N, J=4, u=2, density_iters=0)
    assert list(obj.N) == [N, N, 1] and list(obj.K) == [2 * N, 2 * N, 1] and obj.nnz == M
    x = rng.standard_normal((N, N, 1, 2)) + 1j * rng.standard_normal((N, N, 1, 2))
    assert rel(obj.fNUFT(x), ref.fNUFT(x)) < TOL_OP
    y = rng.standard_normal((M, 2)) + 1j * rng.standard_normal((M, 2))
    assert rel(obj.aNUFT(y), ref.aNUFT(y)) < TOL_OP


def test_all_samples_out_of_bounds(cuda):
    om = np.full((3, 100), 40.0)
    obj = nufft_3d(om, 16, "J", 6)
    assert obj.nnz == 0
    x = np.ones((16, 16, 16), dtype=np.complex64)
    assert np.all(obj.fNUFT(x) == 0)
    assert np.all(obj.aNUFT(np.ones(100, dtype=np.complex64)) == 0)


def test_user_density_and_weights(cuda):
    rng = np.random.default_rng(5)
    N, M = 16, 2000
    om = rng.uniform(-N / 2, N / 2 - 1, size=(3, M))
    d = rng.uniform(0.5, 1.5, M)
    obj = nufft_3d(om, N, "J", 6, "d", d)
    ref = NufftRef(om, N, J=6, d=d)
    np.testing.assert_allclose(obj.d, ref.d.astype(np.float32), rtol=1e-7)
    raw = rng.standard_normal((M, 1)) + 1j * rng.standard_normal((M, 1))
    W = rng.uniform(0, 2, M)
    im = obj.iNUFT(raw, 6, 0.05, W, solver="minres", tol=0)
    imr = ref.iNUFT(raw, 6, 0.05, W, solver="minres", tol=0)
    assert rel(im, imr) < TOL_IMG


def test_minres_tolerance_stop(cuda):
    rng = np.random.default_rng(6)
    N, M = 16, 3000
    om = rng.uniform(-N / 2, N / 2 - 1, size=(3, M))
    obj = nufft_3d(om, N, "J", 6)
    ref = NufftRef(om, N, J=6)
    raw = rng.standard_normal((M, 2)) + 1j * rng.standard_normal((M, 2))
    im, its = obj.iNUFT(raw, 200, 0.1, return_iters=True)
    imr = ref.iNUFT(raw, 200, 0.1)
    assert all(abs(a - b) <= 1 for a, b in zip(its, ref.last_iters)), (its, ref.last_iters)
    assert max(its) < 200
    assert rel(im, imr) < 1e-3


@pytest.mark.parametrize("N,nc", [((64, 96, 160), 2), ((128, 192, 32), 1), ((160, 64, 128), 3)])
def test_fft_lengths_non_cubic(cuda, N, nc):
    """Oversampled lengths K = 128, 192, 256, 320, 384 on every axis and pass
    (register four-step and shared-memory Stockham line FFTs), non-cubic N."""
    torch = cuda
    rng = np.random.default_rng(sum(N) + nc)
    M = 3000
    om = np.vstack([rng.uniform(-n / 2, n / 2 - 1, M) for n in N])
    obj = nufft_3d(om, np.array(N), "J", 6, density_iters=0)
    ref = NufftRef(om, np.array(N), J=6, density_iters=0)
    assert list(obj.K) == [2 * n for n in N]
    x = rng.standard_normal(tuple(N) + (nc,)) + 1j * rng.standard_normal(tuple(N) + (nc,))
    y = rng.standard_normal((M, nc)) + 1j * rng.standard_normal((M, nc))
    assert rel(k_from_dev(obj.fNUFT(img_to_dev(torch, x))), ref.fNUFT(x)) < TOL_OP
    assert rel(img_from_dev(obj.aNUFT(k_to_dev(torch, y))), ref.aNUFT(y)) < TOL_OP


@pytest.mark.parametrize("solver", ["minres", "cg"])
def test_warm_start_matches_oracle(cuda, solver):
    """nufft3d_inverse_x0 (host and device pointers) against the oracle started
    from the same x0, fixed iteration count."""
    torch = cuda
    rng = np.random.default_rng(12)
    N, M = 16, 3000
    om = rng.uniform(-N / 2, N / 2 - 1, size=(3, M))
    obj = nufft_3d(om, N, "J", 6)
    ref = NufftRef(om, N, J=6)
    raw = rng.standard_normal((M, 2)) + 1j * rng.standard_normal((M, 2))
    x0 = ref.iNUFT(raw, 3, 0.1, solver=solver, tol=0)
    imr = ref.iNUFT(raw, 5, 0.1, solver=solver, tol=0, x0=x0)
    im = obj.iNUFT(raw, 5, 0.1, solver=solver, tol=0, x0=x0)
    assert rel(im, imr) < TOL_IMG
    imd = img_from_dev(obj.iNUFT(k_to_dev(torch, raw), 5, 0.1, solver=solver, tol=0, x0=img_to_dev(torch, x0)))
    assert rel(imd, imr) < TOL_IMG
    # warm start from the converged answer stops at once with tol > 0
    xs = ref.iNUFT(raw, 200, 0.1, solver=solver, tol=1e-10)
    _, its = obj.iNUFT(raw, 50, 0.1, solver=solver, tol=1e-3, x0=xs, return_iters=True)
    assert max(its) <= 2


def test_discrep_matches_oracle(cuda):
    """discrep.m: 20 damp updates with warm-started MINRES solves."""
    from oracle.nufft_ref import discrep as discrep_ref
    rng = np.random.default_rng(13)
    N, M = 16, 4000
    om = rng.uniform(-N / 2, N / 2 - 1, size=(3, M))
    obj = nufft_3d(om, N, "J", 6)
    ref = NufftRef(om, N, J=6)
    x = synth.phantom_with_phase(N)
    data = ref.fNUFT(x)[:, 0]
    sd = 0.05 * float(np.std(np.abs(data)))
    data = data + sd * (rng.standard_normal(M) + 1j * rng.standard_normal(M)) / math.sqrt(2)
    d_gpu = obj.discrep(data, sd)
    d_ref = discrep_ref(ref, data, sd)
    assert abs(d_gpu - d_ref) / d_ref < 1e-2, (d_gpu, d_ref)


def test_phase_constraint_matches_oracle(cuda):
    """iNUFT 'phase-constraint' (iNUFT.m:140-168, pprojection nufft_3d.m:325-334)
    on a phantom with smooth phase, host and device paths, fixed iteration
    counts.  Tolerance 1e-3: the phase map is taken from the FP32 MINRES image,
    and voxels where the 3x3 box sum is near zero carry FP32-sized phase
    differences into the second solve."""
    torch = cuda
    N = 16
    om = synth.koosh_ball(N, 16, 600)
    obj = nufft_3d(om, N, "J", 6)
    ref = NufftRef(om, N, J=6)
    x = synth.phantom_with_phase(N)
    raw = np.concatenate([ref.fNUFT(x), ref.fNUFT(x * np.exp(0.3j))], axis=1)
    imr = ref.iNUFT_phase(raw, 6, 0.05, 0.5, tol=0)
    im = obj.iNUFT(raw, 6, 0.05, constraint="phase-constraint", lam=0.5, tol=0)
    assert rel(im, imr) < 1e-3
    imd = img_from_dev(obj.iNUFT(k_to_dev(torch, raw), 6, 0.05, constraint="phase-constraint", lam=0.5, tol=0))
    assert rel(imd, im) < 1e-5
    with pytest.raises(ValueError):
        obj.iNUFT(raw, 6, 0.05, constraint="phase-constraint")      # lambda required
    with pytest.warns(UserWarning):
        plain = obj.iNUFT(raw, 1, 0.05, constraint="phase-constraint", lam=0.5, tol=0)
    assert rel(plain, obj.iNUFT(raw, 1, 0.05, tol=0)) < 1e-6


@pytest.mark.slow
def test_N192_grid_cg_matches_oracle(cuda):
    """N=192 grid (K=384^3 four-step FFTs, 16 coils per plan) with a
    reduced koosh ball (384 x 3000 spokes): 5 CG iterations (tol 0) of coil 0
    against the FP64 oracle CG on the same density (taken from the plan, so
    the oracle skips its 20 density sweeps)."""
    torch = cuda
    N = 192
    om = synth.koosh_ball(N, 384, 3000)
    obj = nufft_3d(om, N, "J", 6)
    ref = NufftRef(om, N, J=6, d=obj.d.astype(np.float64), matrix=False, workers=os.cpu_count())
    rng = np.random.default_rng(14)
    raw = (rng.standard_normal((obj.M, 16)) + 1j * rng.standard_normal((obj.M, 16))).astype(np.complex64)
    im = img_from_dev(obj.iNUFT(k_to_dev(torch, raw), 5, 1e-3, solver="cg", tol=0))
    imr = ref.iNUFT(raw[:, :1], 5, 1e-3, solver="cg", tol=0)
    assert rel(im[..., :1], imr) < TOL_IMG


def test_host_entry_points_pinned_and_pageable_agree(cuda):
    """nufft3d_forward_host / _adjoint_host read and write page-locked buffers
    in place (kernels on mapped host memory) and stage pageable ones; both
    give the device-pointer results."""
    import ctypes
    from nufft_3d_gb300 import _lib
    torch = cuda
    rng = np.random.default_rng(15)
    N, M, nc = 32, 20000, 4
    om = rng.uniform(-N / 2, N / 2 - 1, size=(3, M))
    obj = nufft_3d(om, N, "J", 6, density_iters=0)
    L = obj._L
    x = torch.randn((nc, N, N, N), dtype=torch.complex64)
    y = torch.randn((nc, M), dtype=torch.complex64)
    k_dev = obj.fNUFT(x.cuda()).cpu()
    a_dev = obj.aNUFT(y.cuda()).cpu()
    for pinned in (True, False):
        xi = x.pin_memory() if pinned else x.clone()
        yi = y.pin_memory() if pinned else y.clone()
        ko = torch.empty((nc, M), dtype=torch.complex64)
        ao = torch.empty((nc, N, N, N), dtype=torch.complex64)
        if pinned:
            ko, ao = ko.pin_memory(), ao.pin_memory()
        _lib.check(L.nufft3d_forward_host(obj.plan, xi.data_ptr(), ko.data_ptr(), nc))
        _lib.check(L.nufft3d_adjoint_host(obj.plan, yi.data_ptr(), ao.data_ptr(), nc))
        assert float((ko - k_dev).abs().max()) == 0.0
        assert float((ao - a_dev).abs().max()) == 0.0
