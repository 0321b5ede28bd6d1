"""CPU tests: the FP64 oracle against independent known answers and the golden fixtures.

The reference ships no tests or golden vectors (it is MATLAB and cannot run
here), so the oracle is pinned by known answers that do not depend on it.
"""
import glob
import math
import os

import numpy as np
import pytest
from scipy.special import i0

from nufft_3d_gb300 import synth
from oracle.interp_ref import interp_adjoint, interp_forward
from oracle.nufft_ref import NufftRef, beatty_alpha, bessi0, kernel, minres, cg

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def test_bessi0_within_abramowitz_stegun_bound():
    # A&S 9.8.1 |eps| < 1.6e-7, 9.8.2 |eps| < 1.9e-7 (relative, on the scaled forms)
    x = np.linspace(0, 30, 3001)
    assert np.max(np.abs(bessi0(x) / i0(x) - 1)) < 2e-7


def test_bessi0_imaginary_argument_small_branch():
    # kernel.m:19-23 with ax = i*b: y = (ax/3.75)^2 = -(b/3.75)^2 (real), same
    # polynomial, no x2 hack; it tracks J0(b) = I0(i b) only near b = 0
    from scipy.special import j0
    b = np.linspace(0, 3.7, 50)
    y = -(b / 3.75) ** 2
    poly = 1 + y * (3.5156229 + y * (3.0899424 + y * (1.2067492 + y * (0.2659732 + y * (0.360768e-1 + y * 0.45813e-2)))))
    np.testing.assert_allclose(bessi0(1j * b).real, poly, rtol=1e-14)
    assert np.all(bessi0(1j * b).imag == 0)
    assert np.max(np.abs(poly[b < 1] - j0(b[b < 1]))) < 1e-6


def test_bessi0_imaginary_large_branch_has_x2_hack():
    # kernel.m:32-34: purely imaginary arguments with |ax| >= 3.75 are doubled
    ax = 1j * np.array([4.0, 10.0])
    a = ax
    y = 3.75 / a
    base = (np.exp(a) / np.sqrt(a)) * (0.39894228 + y * (0.1328592e-1 + y * (0.225319e-2 + y * (-0.157565e-2 + y * (
        0.916281e-2 + y * (-0.2057706e-1 + y * (0.2635537e-1 + y * (-0.1647633e-1 + y * 0.392377e-2))))))))
    np.testing.assert_allclose(bessi0(ax), 2 * base, rtol=1e-14)


def test_beatty_alpha_known_values():
    # nufft_3d.m:87,90 at J=6, u=2
    assert beatty_alpha(6, 2, True) == pytest.approx(13.711891329818519, abs=1e-12)
    assert beatty_alpha(6, 2, False) == pytest.approx(13.855100346124816, abs=1e-12)


def test_kernel_endpoints():
    a = beatty_alpha(6, 2, True)
    w = kernel([0.0, 9.0], a, 6)
    assert w[0] == pytest.approx(1.0, abs=1e-15)
    assert w[1] == pytest.approx(1.0 / bessi0(np.array([a]))[0], rel=1e-12)


@pytest.mark.parametrize("J,radial", [(6, True), (4, True), (6, False)])
def test_forward_matches_nudft_scaled(J, radial):
    rng = np.random.default_rng(1)
    N, M = 16, 3000
    om = rng.uniform(-N / 2, N / 2 - 1, size=(3, M))
    ref = NufftRef(om, N, J=J, u=2, radial=radial, density_iters=0)
    x = rng.standard_normal((N, N, N)) + 1j * rng.standard_normal((N, N, N))
    k = ref.fNUFT(x)[:, 0]
    kd = ref.nudft(x)[:, 0] / math.sqrt(ref.nnz)
    err = np.linalg.norm(k - kd) / np.linalg.norm(kd)
    assert err < (3e-3 if J == 4 else 1e-4), err


def test_adjoint_identity_exact():
    rng = np.random.default_rng(2)
    N, M = 16, 2500
    om = rng.uniform(-N / 2, N / 2 - 1, size=(3, M))
    ref = NufftRef(om, N, J=6, u=2, density_iters=0)
    x = rng.standard_normal((N, N, N)) + 1j * rng.standard_normal((N, N, N))
    y = rng.standard_normal(M) + 1j * rng.standard_normal(M)
    lhs = np.vdot(y, ref.fNUFT(x)[:, 0])
    rhs = np.vdot(ref.aNUFT(y).reshape(-1, order="F"), x.reshape(-1, order="F"))
    assert abs(lhs - rhs) / abs(lhs) < 1e-12


def test_cartesian_full_grid_is_scaled_dft_and_density_one():
    # test_nufft3d.m:46-52 Cartesian trajectory: fNUFT reduces to a DFT, d = 1
    N = 12
    g = np.arange(-N // 2, N // 2)
    kx, ky, kz = np.meshgrid(g, g, g, indexing="ij")
    om = np.stack([kx.ravel(order="F"), ky.ravel(order="F"), kz.ravel(order="F")]).astype(float)
    ref = NufftRef(om, N, J=6, u=2, density_iters=20)
    assert ref.nnz == N ** 3
    np.testing.assert_allclose(ref.d, 1.0, atol=1e-12)
    rng = np.random.default_rng(0)
    x = rng.standard_normal((N, N, N)) + 1j * rng.standard_normal((N, N, N))
    k = ref.fNUFT(x)[:, 0] * math.sqrt(ref.nnz)
    dft = ref.nudft(x)[:, 0]
    assert np.linalg.norm(k - dft) / np.linalg.norm(dft) < 1e-4


def test_deap_matches_analytic_lewitt():
    # the analytic branch kept disabled in deap.m:38-95 (radial, not centered)
    rng = np.random.default_rng(0)
    om = rng.uniform(-8, 7, size=(3, 100))
    ref = NufftRef(om, 16, J=6, u=2, density_iters=0)
    a, alpha = ref.J / 2, ref.alpha
    xs = [(np.arange(ref.N[j]) - ref.N[j] / 2) / ref.K[j] for j in range(3)]
    X, Y, Z = np.meshgrid(*xs, indexing="ij")
    R = np.sqrt(X ** 2 + Y ** 2 + Z ** 2)
    C = 4 * math.pi * a ** 3 / i0(alpha)
    U = np.zeros_like(R)
    k = 2 * math.pi * a * R < alpha
    s = np.sqrt(alpha ** 2 - (2 * math.pi * a * R[k]) ** 2)
    U[k] = C * (np.cosh(s) / s ** 2 - np.sinh(s) / s ** 3)
    s = np.sqrt((2 * math.pi * a * R[~k]) ** 2 - alpha ** 2)
    U[~k] = C * (np.sin(s) / s ** 3 - np.cos(s) / s ** 2)
    assert np.linalg.norm(ref.U - 1 / U) / np.linalg.norm(1 / U) < 1e-5


def test_diag_qq_close_to_one():
    # density.m:44-82 diagnostics: diag(Q'Q) ~ 1 and diag(Q'DQ) ~ 1
    om = synth.koosh_ball(16, 16, 400)
    ref = NufftRef(om, 16, J=6, u=2, density_iters=20)
    N = 16
    for j in [0, 7 + 16 * 8 + 256 * 8]:
        e = np.zeros(N ** 3, dtype=complex)
        e[j] = 1
        e = e.reshape((N, N, N), order="F")
        assert abs(ref.iprojection(e, 0, 1)[j, 0] - 1) < 1e-3      # Q'Q
        assert abs(ref.iprojection(e, 0, ref.d)[j, 0] - 1) < 1e-3  # Q'DQ


def test_matrix_free_c_oracle_equals_sparse():
    rng = np.random.default_rng(0)
    for opts in (dict(J=6, u=2, radial=True), dict(J=5, u=1.5, radial=False), dict(J=3, u=2, radial=True)):
        om = rng.uniform(-9, 8, size=(3, 1500))
        ref = NufftRef(om, 16, density_iters=0, **opts)
        G = int(np.prod(ref.K))
        g = rng.standard_normal((G, 2)) + 1j * rng.standard_normal((G, 2))
        y = rng.standard_normal((ref.M, 2)) + 1j * rng.standard_normal((ref.M, 2))
        np.testing.assert_allclose(interp_forward(ref, g), ref.H @ g, rtol=0, atol=1e-12)
        np.testing.assert_allclose(interp_adjoint(ref, y), ref.H.T @ y, rtol=0, atol=1e-12)


def test_two_d_case_keeps_every_point():
    # nufft_3d.m:104-106,125: om(3,:)==0 -> N3 = 1, K3 = 1 and all points in bounds
    rng = np.random.default_rng(0)
    om = np.vstack([rng.uniform(-20, 20, (2, 300)), np.zeros((1, 300))])
    ref = NufftRef(om, 16, J=4, u=2, density_iters=0)
    assert ref.N[2] == 1 and ref.K[2] == 1 and ref.nnz == 300


def test_argument_errors_match_reference():
    om = np.zeros((3, 10))
    with pytest.raises(ValueError):
        NufftRef(np.zeros((2, 10)), 16)
    with pytest.raises(ValueError):
        NufftRef(om + 1, 15)
    with pytest.raises(ValueError):
        NufftRef(om + 1, 16, u=0.5)


def test_solvers_on_spd_matrix():
    rng = np.random.default_rng(0)
    n = 40
    B = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    A = B.conj().T @ B + np.eye(n)
    b = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    xe = np.linalg.solve(A, b)
    for solver in (minres, cg):
        x, it = solver(lambda v: A @ v, b, 0, 200)
        assert np.linalg.norm(x - xe) / np.linalg.norm(xe) < 1e-8
    x, it = minres(lambda v: A @ v, b, 1e-4, 500)
    assert np.linalg.norm(A @ x - b) / np.linalg.norm(b) <= 1.01e-4


@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(GOLDEN, "*.npz"))))
def test_golden_fixtures_reproduce(path):
    z = np.load(path)
    ref = NufftRef(z["om"], int(z["N"]), J=float(z["J"]), u=float(z["u"]), radial=bool(z["radial"]))
    assert ref.nnz == int(z["nnz"])
    k = ref.fNUFT(z["x"].astype(np.complex128))
    assert np.linalg.norm(k - z["k"]) / np.linalg.norm(z["k"]) < 1e-6
    a = ref.aNUFT(z["y"].astype(np.complex128))
    assert np.linalg.norm(a - z["a"]) / np.linalg.norm(z["a"]) < 1e-6
    np.testing.assert_allclose(ref.U, z["U"], rtol=1e-6)
    np.testing.assert_allclose(ref.d, z["d"], rtol=1e-5, atol=1e-6)


def test_warm_start_solvers():
    """minres/cg from x0: the exact solution stops at once; any x0 reaches the
    same solution; the stop test stays relative to |b| (MATLAB semantics)."""
    from oracle.nufft_ref import cg, minres
    rng = np.random.default_rng(11)
    n = 40
    Q = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    H = Q @ Q.conj().T + n * np.eye(n)
    b = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    A = lambda v: H @ v
    xs = np.linalg.solve(H, b)
    for solver in (minres, cg):
        x, it = solver(A, b, 1e-10, 200, xs)
        assert it <= 1 and np.allclose(x, xs)
        x0 = rng.standard_normal(n) + 1j * rng.standard_normal(n)
        x, _ = solver(A, b, 1e-12, 200, x0)
        assert np.linalg.norm(x - xs) / np.linalg.norm(xs) < 1e-9
