"""Transform lengths with a prime factor of 17 or more (Bluestein's algorithm in
the run-time kernels) against the oracle: single solves in FP64 and FP32 on
every boundary family, and a batch that mixes them with other lengths."""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12
FP32_TOL = 5e-6

# padded lengths: 17, 19, 23 (periodic); 74 = 2 x 37, 34 = 2 x 17 (unbounded);
# 29 periodic with 2 x 31 unbounded; 97 periodic
CASES = [
    ((17, 19, 23), (1, 1, 1), dict(curl=True)),
    ((37, 10, 17), (0, 0, 0), dict()),
    ((29, 29, 31), (1, 1, 0), dict(div=True)),
    ((12, 41, 19), (0, 0, 1), dict(grad=True)),
    ((97, 8, 6), (1, 1, 1), dict()),
]


def _fields(nc, opts, seed, zero_mean):
    rng = np.random.default_rng(seed)
    shape = (nc[2], nc[1], nc[0])
    comps = (0,) if opts.get("grad") else (0, 1, 2)
    out = []
    for c in range(3):
        if c not in comps:
            out.append(None)
            continue
        f = rng.standard_normal(shape)
        if zero_mean:
            f -= f.mean(axis=(1, 2), keepdims=True)
        out.append(f)
    return out


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("ci", range(len(CASES)))
def test_bluestein_lengths_vs_oracle(native, oracle, ci, precision):
    nc, bc, opts = CASES[ci]
    dx = (1.0 / nc[0], 1.3 / nc[1], 0.9 / nc[2])
    B = _fields(nc, opts, 40 + ci, zero_mean=bc == (1, 1, 0))
    ref, _ = oracle.solve3d(nc, bc, dx, B, 2, **opts)
    got, _ = native.solve(nc, bc, dx, B, 2, precision=precision, **opts)
    assert rel_l2(got, ref) < (FP64_TOL if precision == "fp64" else FP32_TOL)


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_bluestein_in_a_batch(native, oracle, precision):
    b = native.PoissonBatch(precision)
    probs = CASES + [((16, 12, 10), (0, 0, 0), dict()), ((9, 13, 11), (1, 1, 1), dict(curl=True))]
    data = []
    for i, (nc, bc, opts) in enumerate(probs):
        b.add(nc, bc, tuple(2.0 / n for n in nc), 2)
        if opts.get("grad"):
            b.set_return_grad(i, True)
        if opts.get("div"):
            b.set_return_div(i, True)
        if opts.get("curl"):
            b.set_return_curl(i, True)
        B = _fields(nc, opts, 70 + i, zero_mean=bc == (1, 1, 0))
        b.push(i, *B)
        data.append(B)
    b.solve()
    tol = FP64_TOL if precision == "fp64" else FP32_TOL
    for i, (nc, bc, opts) in enumerate(probs):
        ref, _ = oracle.solve3d(nc, bc, tuple(2.0 / n for n in nc), data[i], 2, **opts)
        shape = (nc[2], nc[1], nc[0])
        A = [np.full(shape, np.nan) for _ in range(3)]
        b.pull(i, *A)
        A = [a if not np.isnan(a).all() else None for a in A]
        assert rel_l2(A, ref) < tol, (i, nc, bc)
    b.close()
