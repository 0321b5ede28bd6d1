"""GPU parity of the stored interpolation matrix (tap table).

The reference builds H once per trajectory (nufft_3d.m:153-212) and applies
H / H' (nufft_3d.m:259-282).  Plans here store H in tile order for the 8-coil
gather passes of fNUFT (and, built from it, H' for the 8-coil spread passes:
tests/test_gpu_spread_tab.py); these tests check the stored path against the
FP64 oracle and against the same plan with the taps evaluated on the fly
(tap_table=0).

Tolerances: relative L2 <= 1e-5 against FP64 (as the other operator tests);
the two gathers agree to <= 1e-6 (they add the same FP32 products in a
different order); the two spreads to <= 5e-6 (the on-the-fly spread
accumulates 32-bit fixed point, about 22 bits per product, H' in FP32).
"""
import numpy as np
import pytest

from nufft_3d_gb300 import nufft_3d, synth
from oracle.nufft_ref import NufftRef

from test_gpu_parity import TOL_OP, TOL_IMG, img_from_dev, img_to_dev, k_from_dev, k_to_dev, rel

pytestmark = pytest.mark.gpu
TOL_SPREAD_FORMS = 5e-6  # stored-H' spread (FP32) against the fixed-point spread


def _pair(om, N, opts, **kw):
    args = sum(([k, v] for k, v in opts.items()), [])
    on = nufft_3d(om, N, *args, density_iters=0, **kw)
    off = nufft_3d(om, N, *args, density_iters=0, tap_table=0, **kw)
    return on, off


@pytest.mark.parametrize("opts,nc", [
    (dict(J=6, u=2, radial=1), 8),
    (dict(J=6, u=2, radial=1), 11),   # one pass from the table, one (4 coils) on the fly
    (dict(J=4, u=2, radial=0), 8),
    (dict(J=5, u=1.5, radial=1), 8),
    (dict(J=2, u=2, radial=1), 9),
])
def test_table_matches_oracle_and_on_the_fly(cuda, opts, nc):
    torch = cuda
    rng = np.random.default_rng(11)
    N, M = 20, 5000
    om = rng.uniform(-N / 2 - 1, N / 2, size=(3, M))  # some out of bounds, many wrapping tiles
    on, off = _pair(om, N, opts)
    assert on.tap_table_bytes > 0 and off.tap_table_bytes == 0
    ref = NufftRef(om, N, density_iters=0, **opts)
    x = rng.standard_normal((N, N, N, nc)) + 1j * rng.standard_normal((N, N, N, nc))
    y = rng.standard_normal((M, nc)) + 1j * rng.standard_normal((M, nc))
    k_on = k_from_dev(on.fNUFT(img_to_dev(torch, x)))
    k_off = k_from_dev(off.fNUFT(img_to_dev(torch, x)))
    assert rel(k_on, ref.fNUFT(x)) < TOL_OP
    assert rel(k_on, k_off) < 1e-6
    assert np.all(k_on[~ref.ok] == 0)
    a_on = img_from_dev(on.aNUFT(k_to_dev(torch, y)))
    a_off = img_from_dev(off.aNUFT(k_to_dev(torch, y)))
    assert rel(a_on, ref.aNUFT(y)) < TOL_OP
    assert rel(a_on, a_off) < TOL_SPREAD_FORMS


def test_table_two_d(cuda):
    torch = cuda
    rng = np.random.default_rng(12)
    N, M, nc = 32, 4000, 8
    om = np.vstack([rng.uniform(-20, 20, (2, M)), np.zeros((1, M))])
    on, off = _pair(om, N, dict(J=6))
    assert on.tap_table_bytes > 0
    ref = NufftRef(om, N, J=6, u=2, density_iters=0)
    x = rng.standard_normal((N, N, 1, nc)) + 1j * rng.standard_normal((N, N, 1, nc))
    assert rel(on.fNUFT(x), ref.fNUFT(x)) < TOL_OP
    y = rng.standard_normal((M, nc)) + 1j * rng.standard_normal((M, nc))
    assert rel(on.aNUFT(y), ref.aNUFT(y)) < TOL_OP
    assert rel(on.aNUFT(y), off.aNUFT(y)) < TOL_SPREAD_FORMS


@pytest.mark.parametrize("spb", [37, 300, 4096])
def test_table_piece_sizes(cuda, spb):
    """Pieces of a few samples per warp up to pieces larger than the default."""
    torch = cuda
    N = 32
    om = synth.koosh_ball(N, 64, 1500)
    on, off = _pair(om, N, dict(J=6), samples_per_block=spb)
    g = torch.Generator(device="cuda").manual_seed(1)
    x = torch.randn((8, N, N, N), dtype=torch.complex64, device="cuda", generator=g)
    y = torch.randn((8, on.M), dtype=torch.complex64, device="cuda", generator=g)
    k_on, k_off = on.fNUFT(x), off.fNUFT(x)
    assert float((k_on - k_off).abs().norm() / k_off.abs().norm()) < 1e-6
    a_on, a_off = on.aNUFT(y), off.aNUFT(y)
    assert float((a_on - a_off).abs().norm() / a_off.abs().norm()) < TOL_SPREAD_FORMS


def test_table_not_built_where_it_does_not_apply(cuda):
    rng = np.random.default_rng(13)
    om = rng.uniform(-8, 7, size=(3, 1000))
    assert nufft_3d(om, 16, "J", 8, density_iters=0).tap_table_bytes == 0          # R = 4
    assert nufft_3d(om, 16, "J", 6, density_iters=0, coils_per_pass=4).tap_table_bytes == 0
    assert nufft_3d(om, 16, "J", 6, density_iters=0, tap_table=1).tap_table_bytes > 0


def test_table_shared_handle_and_solver(cuda):
    """A shared handle uses the same stored H; CG on 8 coils matches the oracle."""
    torch = cuda
    N = 32
    om = synth.koosh_ball(N, 64, 1200)
    obj = nufft_3d(om, N, "J", 6)
    assert obj.tap_table_bytes > 0
    ref = NufftRef(om, N, J=6, u=2, matrix=False)
    rng = np.random.default_rng(14)
    x = rng.standard_normal((N, N, N, 8)) + 1j * rng.standard_normal((N, N, N, 8))
    kr = ref.fNUFT(x)
    h = obj.share()
    try:
        k1 = k_from_dev(obj.fNUFT(img_to_dev(torch, x)))
        k2 = k_from_dev(h.fNUFT(img_to_dev(torch, x)))
        assert np.array_equal(k1, k2)
        assert rel(k1, kr) < TOL_OP
        im = obj.iNUFT(kr, 10, 1e-3, solver="cg", tol=0)
        imr = ref.iNUFT(kr, 10, 1e-3, solver="cg", tol=0)
        assert rel(im, imr) < TOL_IMG
    finally:
        h.close()
