"""GPU tests of the plan-time autotuner (nufft3d_plan_tune).

The tuner changes only how the interpolation is blocked (piece size, coils
per pass), so fNUFT/aNUFT after tuning stay within the operator tolerance of
the FP64 oracle and close to the untuned plan: the forward within 1e-6, the
adjoint within 5e-6 (the spread's per-piece fixed-point scales, and the order
of the grid's float atomics, follow the pieces).  A second plan of the same shape takes the cached choice; handles
shared from a tuned plan, and batches built on it, use its pieces.
"""
import numpy as np
import pytest

from nufft_3d_gb300 import NufftBatch, nufft_3d, synth
from oracle.nufft_ref import NufftRef

pytestmark = pytest.mark.gpu
TOL_OP = 1e-5
TOL_RETILE = 5e-6  # adjoint after re-piecing: the spread's per-piece fixed-point scales change


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b)))


def test_tune_keeps_results_and_caches(cuda):
    torch = cuda
    N, nc = 40, 8
    om = synth.koosh_ball(N, 40, 2500)
    obj = nufft_3d(om, N, "J", 6, density_iters=0)
    rng = np.random.default_rng(8)
    x = (rng.standard_normal((N, N, N, nc)) + 1j * rng.standard_normal((N, N, N, nc))).astype(np.complex64)
    y = (rng.standard_normal((obj.M, nc)) + 1j * rng.standard_normal((obj.M, nc))).astype(np.complex64)
    k0, a0 = obj.fNUFT(x), obj.aNUFT(y)
    r = obj.tune(nc, force=True)
    assert r["samples_per_block"] in (1024, 2048, 4096)
    assert r["coils_per_pass"] in (2, 4, 8)
    assert r["candidates"] >= 6 and not r["from_cache"]
    assert 0 < r["ms_best"] <= r["ms_default"] * 1.0001
    k1, a1 = obj.fNUFT(x), obj.aNUFT(y)
    assert rel(k1, k0) < 1e-6 and rel(a1, a0) < TOL_RETILE
    ref = NufftRef(om, N, J=6, density_iters=0)
    assert rel(k1, ref.fNUFT(x)) < TOL_OP and rel(a1, ref.aNUFT(y)) < TOL_OP
    # a second plan of the same shape takes the cached choice
    other = nufft_3d(synth.koosh_ball(N, 40, 2500) * 0.999, N, "J", 6, density_iters=0)
    r2 = other.tune(nc)
    assert r2["from_cache"] and (r2["samples_per_block"], r2["coils_per_pass"]) == \
        (r["samples_per_block"], r["coils_per_pass"])
    # a handle shared from the tuned plan keeps working after the plan is gone
    h = obj.share()
    obj.close()
    assert rel(h.fNUFT(x), k1) < 1e-6
    h.close()


def test_batch_on_tuned_plans(cuda):
    torch = cuda
    N, nc = 32, 4
    objs = [nufft_3d(synth.koosh_ball(N, 32, 900 + 100 * i), N, "J", 6, density_iters=0) for i in range(2)]
    for o in objs:
        o.tune(nc, force=True)
    g = torch.Generator(device="cuda").manual_seed(2)
    xs = [torch.randn((nc, N, N, N), dtype=torch.complex64, device="cuda", generator=g) for _ in objs]
    single = [o.fNUFT(x) for o, x in zip(objs, xs)]
    b = NufftBatch(objs, [nc, nc])
    ks = b.forward(xs)
    for k, s in zip(ks, single):
        assert float((k - s).abs().norm() / s.abs().norm()) < 1e-6
    b.close()
