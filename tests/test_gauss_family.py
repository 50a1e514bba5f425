"""The Gaussian-regularised kernel family (an extension with no reference
counterpart), on the CPU: the oracle's kernels against quadratures of their
spectrum zeta_m(s|k|)/|k|^2, and the oracle's solves against closed-form
solutions on every domain. There is no reference parity to pin; these
analytic checks pin the oracle the GPU tests compare with."""
import numpy as np
import pytest
from scipy import integrate, special

import gauss_analytic as ga

S = 0.1


@pytest.mark.parametrize("m", [1, 2, 3, 4])
def test_kernels_match_spectrum_quadrature(oracle, m):
    g = oracle.gauss_green
    kmax = 60 / S
    z = lambda k: ga.zeta(k, m, S)
    for r in (0.013, 0.05, 0.1, 0.17, 0.3, 0.6):
        # 3D: G(r) = (1/(2 pi^2 r)) int zeta(k) sin(kr)/k dk
        q3 = integrate.quad(lambda k: z(k) * np.sin(k * r) / k, 0, kmax, limit=2000, epsabs=1e-14)[0]
        assert abs(q3 / (2 * np.pi ** 2 * r) - g(3, m, S, r)) < 1e-13 * abs(g(3, m, S, r))
        # 2D: G(r) - G(r0) = (1/2pi) int zeta(k) (J0(kr) - J0(k r0))/k dk
        q2 = integrate.quad(lambda k: z(k) * (special.j0(k * r) - special.j0(k * 0.2)) / k, 0, kmax,
                            limit=4000, epsabs=1e-14)[0] / (2 * np.pi)
        assert abs(q2 - (g(2, m, S, r) - g(2, m, S, 0.2))) < 1e-13
        # 1D: G(z) - G(0) = (1/pi) int zeta(k) (cos kz - 1)/k^2 dk
        q1 = integrate.quad(lambda k: z(k) * (np.cos(k * r) - 1) / k ** 2 if k > 0 else -0.5 * r * r, 0, kmax,
                            limit=2000, epsabs=1e-14)[0] / np.pi
        assert abs(q1 - (g(1, m, S, r) - g(1, m, S, 0.0))) < 1e-13


@pytest.mark.parametrize("m", [1, 2, 5])
def test_kernels_tend_to_free_space(oracle, m):
    g = oracle.gauss_green
    for R in (2.0, 5.0):
        assert abs(g(3, m, S, R) - 1 / (4 * np.pi * R)) < 1e-15
        assert abs(g(2, m, S, R) + np.log(R) / (2 * np.pi)) < 1e-15
        assert abs(g(1, m, S, R) + R / 2) < 1e-15
    # the origin is the limit of small r
    for d in (1, 2, 3):
        assert abs(g(d, m, S, 1e-7) - g(d, m, S, 0.0)) < 1e-9 * abs(g(d, m, S, 0.0)) + 1e-12


@pytest.mark.parametrize("bc", [(0, 0, 0), (1, 1, 0), (0, 0, 1), (1, 1, 1)])
@pytest.mark.parametrize("m", [1, 3])
def test_oracle_3d_matches_closed_form(oracle, bc, m):
    n = 32
    B, A_ex, RB_ex = ga.case3d(oracle.gauss_green, bc, n, m)
    h = ga.L_BOX / n
    A, RB = oracle.solve3d((n, n, n), bc, (h, h, h), [B, None, None], reg=2 * m, gauss_width=0.0,
                           want_rhs=True)
    assert np.abs(A[0] - A_ex).max() < 5e-14 * np.abs(A_ex).max()
    if RB_ex is not None:
        # the returned right-hand side is the source filtered by zeta_m
        assert np.abs(RB[0] - RB_ex).max() < 5e-14 * np.abs(RB_ex).max()


@pytest.mark.parametrize("bc", [(0, 0), (1, 1), (0, 1), (1, 0)])
def test_oracle_2d_matches_closed_form(oracle, bc):
    n, m = 64, 2
    B, A_ex = ga.case2d(oracle.gauss_green, bc, n, m)
    h = ga.L_BOX / n
    A, _ = oracle.solve2d((n, n), bc, (h, h), [B, None, None], reg=2 * m, gauss_width=0.0)
    assert np.abs(A[0] - A_ex).max() < 5e-14 * np.abs(A_ex).max()


def test_order_and_width(oracle):
    """reg 0 and 2 give the same (order 2) family; an explicit width equal to
    2h is the default; a negative width is rejected."""
    n = 16
    h = ga.L_BOX / n
    B, _, _ = ga.case3d(oracle.gauss_green, (0, 0, 0), n, 1)
    a0, _ = oracle.solve3d((n, n, n), (0, 0, 0), (h, h, h), [B, None, None], reg=0, gauss_width=0.0)
    a2, _ = oracle.solve3d((n, n, n), (0, 0, 0), (h, h, h), [B, None, None], reg=1, gauss_width=2 * h)
    assert np.array_equal(a0[0], a2[0])
    with pytest.raises(ValueError):
        oracle.solve3d((n, n, n), (0, 0, 0), (h, h, h), [B, None, None], gauss_width=-1.0)


@pytest.mark.parametrize("gauss_width", [None, 0.0])
def test_reprojected_rhs_is_divergence_free(oracle, gauss_width):
    """Periodic domain, reprojection on: the returned right-hand side r
    satisfies k . r_hat = 0 (r = zeta B + ik G (ik . zeta B) with G = 1/|k|^2
    for the reference's kernels, or the family's kernel applied to B),
    whichever kernel family built it. The unpaired Nyquist planes are left
    out: there the reference multiplies by ik and keeps the real part, which
    no exact derivative does (solve3d.cpp:388-437)."""
    n = (16, 12, 10)
    L = (1.0, 0.8, 0.9)
    dx = tuple(L[d] / n[d] for d in range(3))
    rng = np.random.default_rng(17)
    B = [rng.standard_normal((n[2], n[1], n[0])) for _ in range(3)]
    _, RB = oracle.solve3d(n, (1, 1, 1), dx, B, reg=4, curl=True, reproject=True, want_rhs=True,
                           gauss_width=gauss_width)
    k = [2 * np.pi * np.fft.fftfreq(n[d], d=dx[d]) for d in range(3)]
    KZ, KY, KX = np.meshgrid(k[2], k[1], k[0], indexing="ij")
    R = [np.fft.fftn(r) for r in RB]
    div = KX * R[0] + KY * R[1] + KZ * R[2]
    keep = np.ones(div.shape, dtype=bool)
    for d, axis in ((0, 2), (1, 1), (2, 0)):
        if n[d] % 2 == 0:
            sel = [slice(None)] * 3
            sel[axis] = n[d] // 2
            keep[tuple(sel)] = False
    scale = max(np.abs(KX * R[0]).max(), np.abs(KY * R[1]).max(), np.abs(KZ * R[2]).max())
    assert np.abs(div[keep]).max() <= 1e-13 * scale


@pytest.mark.parametrize("gauss_width", [None, 0.0])
def test_periodic_solve_commutes_with_grid_shifts(oracle, gauss_width):
    """On a periodic domain the solve commutes with a cyclic shift of the
    grid, for either kernel family and any output option."""
    n, dx = (12, 10, 8), (0.1, 0.12, 0.15)
    rng = np.random.default_rng(23)
    B = [rng.standard_normal((n[2], n[1], n[0])) for _ in range(3)]
    shift = (3, -2, 5)  # (z, y, x) rolls
    Bs = [np.roll(b, shift, axis=(0, 1, 2)) for b in B]
    for opts in (dict(), dict(curl=True), dict(grad=True)):
        A, _ = oracle.solve3d(n, (1, 1, 1), dx, B, reg=2, gauss_width=gauss_width, **opts)
        As, _ = oracle.solve3d(n, (1, 1, 1), dx, Bs, reg=2, gauss_width=gauss_width, **opts)
        for a, s in zip(A, As):
            assert np.abs(np.roll(a, shift, axis=(0, 1, 2)) - s).max() <= 1e-12 * np.abs(a).max()
