"""GPU parity of the spread from the stored transpose H' (aNUFT's spmv_t,
nufft_3d.m:274-282, from the H built at nufft_3d.m:153-212).

Plans with the stored H also store H' per tile piece (each grid point's row
of samples and weights); the 8-coil spread passes read it and accumulate in
FP32.  These tests compare it with the FP64 oracle (relative L2 <= 1e-5, as
the other operator tests; it measures near 1e-7) and with the same plan's
spread evaluating the kernel (spread_table=0), which accumulates 32-bit fixed
point with about 22 bits per product: the two agree to 5e-6.
"""
import numpy as np
import pytest

from nufft_3d_gb300 import nufft_3d, synth
from oracle.nufft_ref import NufftRef

from test_gpu_parity import TOL_OP, TOL_IMG, img_from_dev, k_to_dev, rel

pytestmark = pytest.mark.gpu
TOL_FORMS = 5e-6  # H' spread (FP32) against the fixed-point spread


def _plans(om, N, opts, **kw):
    args = sum(([k, v] for k, v in opts.items()), [])
    on = nufft_3d(om, N, *args, density_iters=0, tap_table=1, spread_table=1, **kw)
    off = nufft_3d(om, N, *args, density_iters=0, tap_table=1, spread_table=0, **kw)
    assert on.spread_table_bytes > 0 and off.spread_table_bytes == 0
    return on, off


@pytest.mark.parametrize("opts,nc", [
    (dict(J=6, u=2, radial=1), 8),
    (dict(J=6, u=2, radial=1), 16),   # two passes from H'
    (dict(J=6, u=2, radial=1), 10),   # one pass from H', one 2-coil pass evaluating the kernel
    (dict(J=4, u=2, radial=0), 8),
    (dict(J=5, u=1.5, radial=1), 8),
    (dict(J=2, u=2, radial=1), 8),
])
def test_spread_table_matches_oracle(cuda, opts, nc):
    torch = cuda
    rng = np.random.default_rng(21)
    N, M = 20, 5000
    om = rng.uniform(-N / 2 - 1, N / 2, size=(3, M))  # some out of bounds, many wrapping tiles
    on, off = _plans(om, N, opts)
    ref = NufftRef(om, N, density_iters=0, **opts)
    y = rng.standard_normal((M, nc)) + 1j * rng.standard_normal((M, nc))
    a_on = img_from_dev(on.aNUFT(k_to_dev(torch, y)))
    a_off = img_from_dev(off.aNUFT(k_to_dev(torch, y)))
    a_ref = ref.aNUFT(y)
    e = rel(a_on, a_ref)
    assert e < TOL_OP, e
    assert rel(a_on, a_off) < TOL_FORMS


def test_spread_table_split_dense_tile(cuda):
    """One tile holding far more samples than a spread piece (2048): its
    pieces' halos overlap completely, and rows are cut between lane groups."""
    torch = cuda
    rng = np.random.default_rng(22)
    N, nc = 32, 8
    dense = rng.uniform(-1.5, 1.5, size=(3, 9000))   # one or two 8^3 tiles of the 64^3 grid
    sparse = rng.uniform(-N / 2, N / 2 - 1, size=(3, 600))
    om = np.hstack([dense, sparse])
    on, off = _plans(om, N, dict(J=6))
    ref = NufftRef(om, N, J=6, u=2, density_iters=0, matrix=False)
    y = rng.standard_normal((om.shape[1], nc)) + 1j * rng.standard_normal((om.shape[1], nc))
    a_on = img_from_dev(on.aNUFT(k_to_dev(torch, y)))
    assert rel(a_on, ref.aNUFT(y)) < TOL_OP
    assert rel(a_on, img_from_dev(off.aNUFT(k_to_dev(torch, y)))) < TOL_FORMS


def test_spread_table_two_d(cuda):
    torch = cuda
    rng = np.random.default_rng(23)
    N, M, nc = 32, 4000, 8
    om = np.vstack([rng.uniform(-20, 20, (2, M)), np.zeros((1, M))])
    on, off = _plans(om, N, dict(J=6))
    ref = NufftRef(om, N, J=6, u=2, density_iters=0)
    y = rng.standard_normal((M, nc)) + 1j * rng.standard_normal((M, nc))
    a_on = img_from_dev(on.aNUFT(k_to_dev(torch, y)))
    assert rel(a_on, ref.aNUFT(y)) < TOL_OP
    assert rel(a_on, img_from_dev(off.aNUFT(k_to_dev(torch, y)))) < TOL_FORMS


def test_spread_table_coil_gains(cuda):
    """FP32 accumulation: each coil keeps its precision whatever the gains of
    the other coils of its pass."""
    torch = cuda
    rng = np.random.default_rng(24)
    N = 24
    om = synth.koosh_ball(N, 48, 600)
    on, _ = _plans(om, N, dict(J=6))
    ref = NufftRef(om, N, J=6, u=2, density_iters=0, matrix=False)
    gains = np.array([1e-4, 1.0, 3e2, 1e-2, 5.0, 1e-3, 1e1, 0.3])
    y = (rng.standard_normal((on.M, 8)) + 1j * rng.standard_normal((on.M, 8))) * gains
    a = img_from_dev(on.aNUFT(k_to_dev(torch, y)))
    ar = ref.aNUFT(y)
    for c in range(8):
        assert rel(a[..., c], ar[..., c]) < TOL_OP, (c, gains[c])


def test_spread_table_shared_handle_and_cg(cuda):
    """A shared handle reads the same H'; CG through it matches the oracle."""
    torch = cuda
    N = 32
    om = synth.koosh_ball(N, 64, 1200)
    obj = nufft_3d(om, N, "J", 6)
    assert obj.spread_table_bytes > 0  # built by default where it fits
    ref = NufftRef(om, N, J=6, u=2, matrix=False)
    rng = np.random.default_rng(25)
    y = rng.standard_normal((obj.M, 8)) + 1j * rng.standard_normal((obj.M, 8))
    h = obj.share()
    try:
        a1 = img_from_dev(obj.aNUFT(k_to_dev(torch, y)))
        a2 = img_from_dev(h.aNUFT(k_to_dev(torch, y)))
        assert rel(a1, a2) < 1e-6  # the grid's vector atomics may add in another order
        assert rel(a1, ref.aNUFT(y)) < TOL_OP
        im = obj.iNUFT(y, 10, 1e-3, solver="cg", tol=0)
        imr = ref.iNUFT(y, 10, 1e-3, solver="cg", tol=0)
        assert rel(im, imr) < TOL_IMG
    finally:
        h.close()


def test_spread_table_not_built_where_it_does_not_apply(cuda):
    rng = np.random.default_rng(26)
    om = rng.uniform(-8, 7, size=(3, 1000))
    assert nufft_3d(om, 16, "J", 6, density_iters=0, tap_table=0).spread_table_bytes == 0  # needs the stored H
    assert nufft_3d(om, 16, "J", 6, density_iters=0, spread_table=0).spread_table_bytes == 0
    assert nufft_3d(om, 16, "J", 8, density_iters=0).spread_table_bytes == 0  # R = 4: no stored H
    obj = nufft_3d(om, 16, "J", 6, density_iters=0, tap_table=1, spread_table=1)
    assert obj.spread_table_bytes > 0
    assert obj.info()["spread_table_bytes"] == obj.spread_table_bytes
