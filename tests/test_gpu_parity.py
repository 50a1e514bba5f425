"""GPU solve vs the oracle and the reference's golden outputs, through the C ABI.

Tolerances: FP64 transforms <= 1e-12 relative L2 (the reference's own twiddle
recurrence drifts by ~1e-14 at these sizes); FP32 transforms <= 5e-6
relative L2 on white-noise sources (every mode excited, the hardest case).
"""
import numpy as np
import pytest

import manufactured as M
from conftest import golden_cases, load_golden, rel_l2

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12
FP32_TOL = 5e-6


@pytest.mark.parametrize("name", golden_cases())
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_golden(native, name, precision):
    g = load_golden(name)
    solve = native.solve if len(g["ncell"]) == 3 else native.solve2d
    A, RB = solve(g["ncell"], g["bc"], g["dx"], g["B"], g["reg"], precision=precision,
                  want_rhs=True, **g["opts"])
    tol = FP64_TOL if precision == "fp64" else FP32_TOL
    assert rel_l2(A, g["A"]) < tol
    assert rel_l2(RB, g["RB"]) < tol


def _fields(nc, comps, seed, zero_mean=False):
    rng = np.random.default_rng(seed)
    out = []
    for c in range(3):
        if c in comps:
            b = rng.standard_normal((nc[2], nc[1], nc[0]))
            if zero_mean:
                b -= b.mean(axis=(1, 2), keepdims=True)
            out.append(b)
        else:
            out.append(None)
    return out


OPS = [dict(), dict(curl=True), dict(div=True), dict(grad=True), dict(curl=True, reproject=True)]
BCS = [(0, 0, 0), (1, 1, 1), (1, 1, 0), (0, 0, 1)]
SIZES = [(16, 16, 16), (12, 20, 10), (9, 7, 13), (32, 8, 24)]


@pytest.mark.parametrize("bc", BCS)
@pytest.mark.parametrize("op", range(len(OPS)))
@pytest.mark.parametrize("size", range(len(SIZES)))
def test_random_vs_oracle(native, oracle, bc, op, size):
    nc = SIZES[size]
    dx = (2.0 / nc[0], 1.7 / nc[1], 2.3 / nc[2])
    opts = OPS[op]
    reg = (0, 2, 6, 3)[(op + size) % 4]
    B = _fields(nc, (0, 1, 2), 100 * op + size, zero_mean=bc == (1, 1, 0))
    ref, rref = oracle.solve3d(nc, bc, dx, B, reg, want_rhs=True, **opts)
    for prec, tol in (("fp64", FP64_TOL), ("fp32", FP32_TOL)):
        got, rgot = native.solve(nc, bc, dx, B, reg, precision=prec, want_rhs=True, **opts)
        assert rel_l2(got, ref) < tol, prec
        assert rel_l2(rgot, rref) < tol, prec


@pytest.mark.parametrize("comps", [(0,), (1,), (0, 2), (0, 1)])
@pytest.mark.parametrize("bc", BCS)
def test_partial_components(native, oracle, comps, bc):
    nc, dx = (10, 12, 14), (0.1, 0.1, 0.1)
    B = _fields(nc, comps, 7, zero_mean=bc == (1, 1, 0))
    ref, _ = oracle.solve3d(nc, bc, dx, B, 2)
    got, _ = native.solve(nc, bc, dx, B, 2)
    assert rel_l2(got, ref) < FP64_TOL
    if 0 in comps:
        # grad with missing components differentiates B_x (the reference would dereference NULL)
        ref, _ = oracle.solve3d(nc, bc, dx, B, 0, grad=True)
        got, _ = native.solve(nc, bc, dx, B, 0, grad=True)
        assert rel_l2(got, ref) < FP64_TOL


@pytest.mark.parametrize("nc", [(1, 1, 1), (1, 8, 6), (5, 1, 7), (6, 9, 1), (2, 2, 2), (3, 5, 7), (23, 19, 11)])
@pytest.mark.parametrize("bc", BCS)
def test_edge_sizes(native, oracle, nc, bc):
    dx = (0.3, 0.2, 0.1)
    B = _fields(nc, (0, 1, 2), sum(nc), zero_mean=bc == (1, 1, 0))
    ref, _ = oracle.solve3d(nc, bc, dx, B, 2, curl=True)
    got, _ = native.solve(nc, bc, dx, B, 2, curl=True)
    # On the smallest grids the exact curl can vanish (every derivative mode is
    # a Nyquist mode); both solves then return rounding noise, so the error is
    # measured against the scale of a unit solve there.
    scale = max(max(float(np.abs(r).max()) for r in ref), 1e-6 * max(dx) ** 2)
    assert max(float(np.abs(g - r).max()) for g, r in zip(got, ref)) <= FP64_TOL * scale


@pytest.mark.parametrize("bc", BCS)
@pytest.mark.parametrize("reg", [0, 2, 7])
def test_kernel_octant_vs_oracle(native, oracle, bc, reg):
    nc, dx = (12, 10, 14), (0.1, 0.13, 0.09)
    g, zeta = oracle.greens3d(nc, bc, dx, reg)
    pz, py, px = g.shape
    want = g.real[: pz // 2 + 1, : py // 2 + 1, : px // 2 + 1].copy()
    if reg:
        want *= zeta[: pz // 2 + 1, : py // 2 + 1, : px // 2 + 1]
    want /= px * py * pz
    with native.PoissonSolver() as ps:
        ps.setup3d(nc, bc, dx, reg)
        got = ps.kernel_octant()
    assert np.abs(got - want).max() <= 1e-13 * np.abs(want).max()


@pytest.mark.parametrize("name", ["unbounded3d", "periodic3d", "mixed_ppf3d", "mixed_ffp3d"])
def test_reference_validation_programs(native, name):
    """The reference's four 3D validation programs, run on the GPU: same printed error."""
    nc, bc, dx, opt, B, sol = M.case(name)
    A, _ = native.solve(nc, bc, dx, B, 0, **{opt: True})
    err = M.printed_error(A, sol, dx)
    known = M.KNOWN_ERRORS[name]
    if known < 1e-14:
        assert err < 1e-14  # round-off level: any FP64 solve agrees only to round-off
    else:
        assert abs(err - known) <= 1e-3 * known
    A32, _ = native.solve(nc, bc, dx, B, 0, precision="fp32", **{opt: True})
    assert rel_l2(A32, A) < 1e-6


def test_gaussian_erf_solution(native):
    """Unbounded scalar Gaussian (sigma = 0.1) on [-1,1]^3 against erf(r/sqrt2 s)/(4 pi r)."""
    from math import erf
    n, s = 64, 0.1
    dx = 2.0 / n
    x = -1.0 + (np.arange(n) + 0.5) * dx
    Z, Y, X = np.meshgrid(x, x, x, indexing="ij")
    r = np.sqrt(X * X + Y * Y + Z * Z)
    B = (2 * np.pi * s * s) ** -1.5 * np.exp(-r * r / (2 * s * s))
    exact = np.vectorize(erf)(r / (np.sqrt(2) * s)) / (4 * np.pi * r)
    A, _ = native.solve((n, n, n), (0, 0, 0), (dx, dx, dx), [B, None, None], 0)
    err = np.sqrt(np.sum((A[0] - exact) ** 2) / np.sum(exact ** 2))
    assert err < 1e-13  # the reference measures 6.1e-14 here


def test_linearity_and_fp32_at_256(native):
    """Size-independent properties at the 256^3 vector case: linearity and FP32 vs FP64."""
    n = 256
    dx = 2.0 / n
    nc = (n, n, n)
    rng = np.random.default_rng(3)
    B1 = [rng.standard_normal((n, n, n)) for _ in range(3)]
    B2 = [rng.standard_normal((n, n, n)) for _ in range(3)]
    a = 0.37
    A1, _ = native.solve(nc, (0, 0, 0), (dx,) * 3, B1, 6, curl=True)
    A2, _ = native.solve(nc, (0, 0, 0), (dx,) * 3, B2, 6, curl=True)
    A3, _ = native.solve(nc, (0, 0, 0), (dx,) * 3, [a * b1 + b2 for b1, b2 in zip(B1, B2)], 6, curl=True)
    assert rel_l2(A3, [a * x + y for x, y in zip(A1, A2)]) < 1e-13
    A1f, _ = native.solve(nc, (0, 0, 0), (dx,) * 3, B1, 6, curl=True, precision="fp32")
    assert rel_l2(A1f, A1) < 1e-6


def test_fp64_y_pass_just_under_48kb_in_a_fresh_process(oracle):
    """A y transform of 1024 points in FP64 at 2 lines a CTA asks for 49 136
    bytes of dynamic shared memory: under 48 KB, but over it with the
    kernel's static shared memory, so the launch must raise the kernel's
    limit itself (in a fresh process nothing else has raised it)."""
    import os
    import subprocess
    import sys

    from conftest import ROOT
    nc, bc = (6, 512, 4), (0, 0, 0)
    code = ("import numpy as np, poisson_solver_gb300 as ps; "
            f"rng = np.random.default_rng(3); B = rng.standard_normal(({nc[2]}, {nc[1]}, {nc[0]})); "
            f"A, _ = ps.solve({nc}, {bc}, (0.1, 0.01, 0.1), [B, None, None], 2, precision='fp64'); "
            "np.save('out.npy', A[0])")
    env = dict(os.environ, PS_LINES_Y="2", PS_TUNE_CACHE="", PYTHONPATH=ROOT)
    import tempfile
    with tempfile.TemporaryDirectory() as d:
        r = subprocess.run([sys.executable, "-c", code], env=env, cwd=d, capture_output=True, text=True, timeout=300)
        assert r.returncode == 0, r.stderr
        got = np.load(os.path.join(d, "out.npy"))
    B = np.random.default_rng(3).standard_normal((nc[2], nc[1], nc[0]))
    ref, _ = oracle.solve3d(nc, bc, (0.1, 0.01, 0.1), [B, None, None], 2)
    assert rel_l2([got], [ref[0]]) < 1e-12
