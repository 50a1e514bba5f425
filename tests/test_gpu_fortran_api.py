"""Fortran-style features of the reference API: one array holding all
components interleaved with ghost offsets (poisson_solver_push.f,
poisson_solver_pull.f) and Gaussian smoothing of the pushed fields
(poisson_solver_smooth3d.f), against separate-array calls and the oracle."""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu

BCS = [(0, 0, 0), (1, 1, 1), (1, 1, 0), (0, 0, 1)]


def _fields(nc, seed):
    rng = np.random.default_rng(seed)
    return [rng.standard_normal((nc[2], nc[1], nc[0])) for _ in range(3)]


@pytest.mark.parametrize("bc", BCS)
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_smooth3d_vs_oracle(native, oracle, bc, precision):
    nc, dx, s = (12, 10, 14), (0.1, 0.12, 0.08), 0.2
    B = _fields(nc, 7)
    want = oracle.smooth3d(nc, bc, dx, B, s)
    ps = native.PoissonSolver()
    ps.setup3d(nc, bc, dx, 0)
    ps.set_precision(precision)
    ps.push(*B)
    ps.smooth3d(s)
    shape = (nc[2], nc[1], nc[0])
    RB = [np.empty(shape) for _ in range(3)]
    ps.pull(None, None, None, *RB)  # reg 0: the returned right-hand side is the smoothed field
    tol = 1e-12 if precision == "fp64" else 5e-6
    assert rel_l2(RB, want) < tol
    # a solve after smoothing solves the smoothed fields
    ps.solve3d()
    A = [np.empty(shape) for _ in range(3)]
    ps.pull(*A)
    ref, _ = oracle.solve3d(nc, bc, dx, want, 0)
    assert rel_l2(A, ref) < (1e-12 if precision == "fp64" else 5e-6)
    ps.close()


def test_smooth3d_periodic_mode_and_errors(native):
    from poisson_solver_gb300 import PSError
    from poisson_solver_gb300 import _lib as L
    n, dx, s = (32, 24, 16), (0.05, 0.1, 0.2), 0.3
    z, y, x = np.meshgrid(np.arange(n[2]) * dx[2], np.arange(n[1]) * dx[1], np.arange(n[0]) * dx[0],
                          indexing="ij")
    k = [2 * np.pi * m / (n[d] * dx[d]) for d, m in enumerate((5, 3, 2))]
    f = np.sin(k[0] * x - k[1] * y + k[2] * z)
    ps = native.PoissonSolver()
    ps.setup3d(n, (1, 1, 1), dx, 0)
    with pytest.raises(PSError) as e:
        ps.smooth3d(s)  # nothing pushed
    assert e.value.status == L.PS_ERR_STATE
    ps.push(f)
    with pytest.raises(PSError) as e:
        ps.smooth3d(-1.0)
    assert e.value.status == L.PS_ERR_ARGUMENT
    ps.smooth3d(s)
    out = np.empty_like(f)
    ps.pull(None, None, None, out)
    want = np.exp(-0.5 * s * s * sum(v * v for v in k)) * f
    assert np.linalg.norm(out - want) <= 1e-13 * np.linalg.norm(f)
    ps.close()


@pytest.mark.parametrize("ncomp,opts", [(1, dict()), (1, dict(grad=True)), (3, dict(curl=True)), (2, dict())])
def test_interleaved_push_pull_with_ghosts(native, ncomp, opts):
    nc, bc, dx, reg = (10, 9, 8), (0, 0, 0), (0.1, 0.11, 0.12), 2
    g = (2, 1, 3)  # ghost offsets (x, y, z)
    ext = (nc[0] + 2 * g[0], nc[1] + 2 * g[1] + 1, nc[2] + 2 * g[2])
    B = _fields(nc, 11)[:ncomp]
    rng = np.random.default_rng(3)
    arr = rng.standard_normal((ext[2], ext[1], ext[0], ncomp))  # ghost cells hold noise
    for c in range(ncomp):
        arr[g[2]:g[2] + nc[2], g[1]:g[1] + nc[1], g[0]:g[0] + nc[0], c] = B[c]
    # separate arrays
    ps = native.PoissonSolver()
    ps.setup3d(nc, bc, dx, reg)
    for k, v in opts.items():
        getattr(ps, "set_return_" + k)(v)
    ps.push(*B, *([None] * (3 - ncomp)))
    ps.solve3d()
    shape = (nc[2], nc[1], nc[0])
    A = [np.full(shape, np.nan) for _ in range(3)]
    RB = [np.full(shape, np.nan) for _ in range(3)]
    ps.pull(*A, *RB)
    # one interleaved array each way
    ps2 = native.PoissonSolver()
    ps2.setup3d(nc, bc, dx, reg)
    for k, v in opts.items():
        getattr(ps2, "set_return_" + k)(v)
    ps2.push_interleaved(arr, offset=g)
    ps2.solve3d()
    a_out = np.full((ext[2], ext[1], ext[0], 3), 7.0)
    b_out = np.full((ext[2], ext[1], ext[0], ncomp), 7.0)
    ps2.pull_interleaved(a_out, b_out, offset=g)
    box = (slice(g[2], g[2] + nc[2]), slice(g[1], g[1] + nc[1]), slice(g[0], g[0] + nc[0]))
    for c in range(3):
        got = a_out[box + (c,)]
        if np.isnan(A[c]).all():
            assert np.all(got == 0.0)  # not produced: written as zero
        else:
            assert np.array_equal(got, A[c])
    for c in range(ncomp):
        assert np.array_equal(b_out[box + (c,)], RB[c])
    # outside the box nothing was written
    mask = np.ones(a_out.shape[:3], dtype=bool)
    mask[box] = False
    assert np.all(a_out[mask] == 7.0) and np.all(b_out[mask] == 7.0)
    ps.close()
    ps2.close()


def test_interleaved_errors_leave_arrays_untouched(native):
    import ctypes

    from poisson_solver_gb300 import _lib as L
    nc, dx = (6, 5, 4), (0.1, 0.1, 0.1)
    ps = native.PoissonSolver()
    ps.setup3d(nc, (0, 0, 0), dx, 0)
    lib, h = ps._lib, ps._h
    dp = ctypes.POINTER(ctypes.c_double)
    ext = (ctypes.c_int * 3)(*nc)
    off = (ctypes.c_int * 3)(0, 0, 0)
    b = np.random.default_rng(5).standard_normal((nc[2], nc[1], nc[0], 1))
    # extents too small for the field at its offset; more than three components
    small = (ctypes.c_int * 3)(nc[0] - 1, nc[1], nc[2])
    assert lib.ps_push_interleaved(h, b.ctypes.data_as(dp), 1, small, off) == L.PS_ERR_ARGUMENT
    assert lib.ps_push_interleaved(h, b.ctypes.data_as(dp), 4, ext, off) == L.PS_ERR_ARGUMENT
    assert lib.ps_push_interleaved(h, b.ctypes.data_as(dp), 1, ext, off) == L.PS_OK
    assert lib.ps_solve3d(h) == L.PS_OK
    # a bad second array: the call fails before writing the first
    a = np.full((nc[2], nc[1], nc[0], 1), 7.0)
    rb = np.zeros((nc[2], nc[1], nc[0], 5))
    assert lib.ps_pull_interleaved(h, a.ctypes.data_as(dp), 1, rb.ctypes.data_as(dp), 5, ext, off) == L.PS_ERR_ARGUMENT
    assert np.all(a == 7.0)
    assert lib.ps_pull_interleaved(h, a.ctypes.data_as(dp), 1, None, 0, ext, off) == L.PS_OK
    assert not np.all(a == 7.0)
    ps.close()
