"""The Gaussian-regularised kernel family on the GPU (an extension with no
reference counterpart): against the oracle on every domain, output option
and precision, against closed-form solutions, and the set_kernel API."""
import numpy as np
import pytest
from scipy import special

import gauss_analytic as ga
from conftest import rel_l2

pytestmark = pytest.mark.gpu

BCS3 = [(0, 0, 0), (1, 1, 0), (0, 0, 1), (1, 1, 1)]
OPTS = {"none": {}, "grad": {"grad": True}, "curl": {"curl": True}, "div": {"div": True}}


def _fields(shape, seed, ncomp=3):
    rng = np.random.default_rng(seed)
    return [rng.standard_normal(shape) for _ in range(ncomp)]


@pytest.mark.parametrize("bc", BCS3)
@pytest.mark.parametrize("opt", list(OPTS))
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_3d_vs_oracle(native, oracle, bc, opt, precision):
    nc, dx, reg, width = (20, 16, 24), (0.05, 0.06, 0.045), 4, 0.13
    B = _fields((nc[2], nc[1], nc[0]), 11)
    kw = OPTS[opt]
    want_A, want_R = oracle.solve3d(nc, bc, dx, B, reg=reg, want_rhs=True, gauss_width=width, **kw)
    got_A, got_R = native.solve(nc, bc, dx, B, reg_order=reg, precision=precision, want_rhs=True,
                                kernel="gaussian", width=width, **kw)
    tol = 1e-12 if precision == "fp64" else 5e-6
    assert rel_l2(got_A, want_A) < tol
    assert rel_l2(got_R, want_R) < tol


def test_3d_reprojection_vs_oracle(native, oracle):
    nc, dx, bc = (16, 18, 14), (0.06, 0.05, 0.07), (0, 0, 0)
    B = _fields((nc[2], nc[1], nc[0]), 5)
    want_A, want_R = oracle.solve3d(nc, bc, dx, B, reg=2, curl=True, reproject=True, want_rhs=True,
                                    gauss_width=0.0)
    got_A, got_R = native.solve(nc, bc, dx, B, reg_order=2, curl=True, reproject=True, want_rhs=True,
                                kernel="gaussian")
    assert rel_l2(got_A, want_A) < 1e-12
    assert rel_l2(got_R, want_R) < 1e-12


@pytest.mark.parametrize("bc", [(0, 0), (1, 1), (0, 1), (1, 0)])
@pytest.mark.parametrize("opt", ["none", "grad", "curl"])
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_2d_vs_oracle(native, oracle, bc, opt, precision):
    nc, dx, reg = (24, 20), (0.05, 0.06), 6
    B = _fields((nc[1], nc[0]), 3)
    kw = OPTS[opt]
    want_A, want_R = oracle.solve2d(nc, bc, dx, B, reg=reg, want_rhs=True, gauss_width=0.0, **kw)
    got_A, got_R = native.solve2d(nc, bc, dx, B, reg_order=reg, precision=precision, want_rhs=True,
                                  kernel="gaussian", **kw)
    tol = 1e-12 if precision == "fp64" else 5e-6
    assert rel_l2(got_A, want_A) < tol
    assert rel_l2(got_R, want_R) < tol


@pytest.mark.parametrize("bc", BCS3)
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_3d_closed_form(native, oracle, bc, precision):
    n, m = 32, 2
    B, A_ex, RB_ex = ga.case3d(oracle.gauss_green, bc, n, m)
    h = ga.L_BOX / n
    A, RB = native.solve((n, n, n), bc, (h, h, h), [B, None, None], reg_order=2 * m, precision=precision,
                         want_rhs=True, kernel="gaussian")
    tol = 1e-13 if precision == "fp64" else 1e-5
    assert np.abs(A[0] - A_ex).max() < tol * np.abs(A_ex).max()
    if RB_ex is not None:
        assert np.abs(RB[0] - RB_ex).max() < tol * np.abs(RB_ex).max()


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_3d_unbounded_closed_form_large(native, precision):
    """128^3 (padded 256^3, the bulk-copy kernels in FP32): a unit Gaussian of
    width s under the order-2 kernel of width 2h is erf(r/(sqrt2 S))/(4 pi r),
    S^2 = (2h)^2 + s^2."""
    n, s = 128, 0.12
    x, h = ga.cell_centres(n)
    Z, Y, X = np.meshgrid(x, x, x, indexing="ij")
    R = np.sqrt(X ** 2 + Y ** 2 + Z ** 2)
    B = np.exp(-R ** 2 / (2 * s * s)) / (2 * np.pi * s * s) ** 1.5
    S = np.hypot(2 * h, s)
    A_ex = special.erf(R / (np.sqrt(2) * S)) / (4 * np.pi * R)
    A, _ = native.solve((n, n, n), (0, 0, 0), (h, h, h), [B, None, None], reg_order=2, precision=precision,
                        kernel="gaussian")
    tol = 1e-13 if precision == "fp64" else 1e-5
    assert np.abs(A[0] - A_ex).max() < tol * np.abs(A_ex).max()


@pytest.mark.parametrize("bc", [(0, 0), (1, 1), (0, 1), (1, 0)])
def test_2d_closed_form(native, oracle, bc):
    n, m = 64, 2
    B, A_ex = ga.case2d(oracle.gauss_green, bc, n, m)
    h = ga.L_BOX / n
    A, _ = native.solve2d((n, n), bc, (h, h), [B, None, None], reg_order=2 * m, kernel="gaussian")
    assert np.abs(A[0] - A_ex).max() < 1e-13 * np.abs(A_ex).max()


def test_set_kernel_api(native):
    nc, dx, bc = (16, 16, 16), (0.1, 0.1, 0.1), (0, 0, 0)
    shape = (16, 16, 16)
    B = _fields(shape, 9, 1)[0]
    ps = native.PoissonSolver()
    ps.setup3d(nc, bc, dx, 2)
    ps.push(B)
    ps.solve3d()
    a_spec = np.empty(shape)
    ps.pull(a_spec)
    # switching the family on a set-up handle rebuilds the kernel, as a new setup
    ps.set_kernel("gaussian")
    with pytest.raises(native.PSError):
        ps.solve3d()  # the pushed fields were dropped
    ps.push(B)
    ps.solve3d()
    a_gauss = np.empty(shape)
    ps.pull(a_gauss)
    assert not np.allclose(a_gauss, a_spec)
    ps.set_kernel("spectral")
    ps.push(B)
    ps.solve3d()
    a_back = np.empty(shape)
    ps.pull(a_back)
    assert np.array_equal(a_back, a_spec)
    lib, h = ps._lib, ps._h
    assert lib.ps_set_kernel(h, 7, 0.0) == native._lib.PS_ERR_ARGUMENT
    assert lib.ps_set_kernel(h, 1, -1.0) == native._lib.PS_ERR_ARGUMENT
    assert lib.ps_set_kernel(h, 1, float("nan")) == native._lib.PS_ERR_ARGUMENT
    assert lib.ps_set_kernel(None, 1, 0.0) == native._lib.PS_ERR_ARGUMENT
    ps.close()
