"""GPU parity of the batched (multi-volume) operators: every volume of a batch
equals its own single-plan fNUFT / aNUFT / CG iNUFT (rel L2 <= 1e-5 for the
operators, <= 1e-4 for the iterative images)."""
import numpy as np
import pytest

from nufft_3d_gb300 import NufftBatch, nufft_3d, synth

pytestmark = pytest.mark.gpu
TOL_OP = 1e-5
TOL_IMG = 1e-4


def rel(a, b):
    return float((a - b).abs().norm() / b.abs().norm())


def volumes():
    specs = [(16, "koosh", 3), (24, "random", 1), (32, "koosh", 8), (20, "spiral", 4), (32, "koosh", 2)]
    out = []
    for i, (N, kind, nc) in enumerate(specs):
        if kind == "koosh":
            om = synth.koosh_ball(N, N, 40 * N)
        elif kind == "random":
            om = synth.random_uniform(N, 3 * N ** 3 // 2, seed=i)
        else:
            om = synth.stack_of_spirals(N, n_interleaves=4, n_samples=256, n_partitions=N)
        out.append((om, N, nc))
    return out


def test_batch_matches_single(cuda):
    torch = cuda
    vols = volumes()
    objs = [nufft_3d(om, N, "J", 6) for om, N, _ in vols]
    objs[4] = objs[2].share() if vols[4][1] == vols[2][1] and vols[4][0].shape == vols[2][0].shape else objs[4]
    ncs = [nc for _, _, nc in vols]
    g = torch.Generator(device="cuda").manual_seed(0)
    xs = [torch.randn((nc,) + (int(o.N[2]), int(o.N[1]), int(o.N[0])), dtype=torch.complex64, device="cuda",
                      generator=g) for o, nc in zip(objs, ncs)]
    ys = [torch.randn((nc, o.M), dtype=torch.complex64, device="cuda", generator=g) for o, nc in zip(objs, ncs)]
    single_k = [o.fNUFT(x) for o, x in zip(objs, xs)]
    single_a = [o.aNUFT(y) for o, y in zip(objs, ys)]
    single_i = [o.iNUFT(y, 8, 0.05, solver="cg", tol=0) for o, y in zip(objs, ys)]
    batch = NufftBatch(objs, ncs)
    ks = batch.forward(xs)
    xa = batch.adjoint(ys)
    xi, its = batch.inverse(ys, 8, 0.05, tol=0, return_iters=True)
    torch.cuda.synchronize()
    for v in range(len(objs)):
        assert rel(ks[v], single_k[v]) < TOL_OP, v
        assert rel(xa[v], single_a[v]) < TOL_OP, v
        assert rel(xi[v], single_i[v]) < TOL_IMG, v
    assert all(i == 8 for i in its)
    batch.close()
    for o in objs:
        o.close()


def test_batch_rejects_mixed_kernels(cuda):
    om = synth.koosh_ball(16, 16, 200)
    a = nufft_3d(om, 16, "J", 6)
    b = nufft_3d(om, 16, "J", 4)
    with pytest.raises(Exception, match="share"):
        NufftBatch([a, a], [1, 1])
    with pytest.raises(Exception, match="kernel"):
        NufftBatch([a, b], [1, 1])
    c = nufft_3d(om, 16, "J", 6, "u", 1.5)   # same ceil(J/2), different alpha
    with pytest.raises(Exception, match="kernel"):
        NufftBatch([a.share(), c], [1, 1])
