"""Rader's algorithm in the run-time transform kernels (FP32 plan variant,
PS_PLAN_* bit 2): a length whose largest prime p divides it once, with p - 1
and the cofactor free of primes above 13, runs a first stage of radix p whose
p-point DFTs are cyclic convolutions of p - 1 points, in place of Bluestein's
two transforms of at least 2 L - 1 points. Each case is checked against the
oracle at the FP32 tolerance, with the stages ps_get_pass_plan reports;
FP64 transforms ignore the variant; batches take it through
ps_batch_set_tuning."""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu

FP32_TOL = 5e-6
RADER = 4


def _fields(nc, seed, ncomp=3):
    rng = np.random.default_rng(seed)
    return [rng.standard_normal((nc[2], nc[1], nc[0])) for _ in range(ncomp)]


def _set_plan(monkeypatch, pv):
    for ax in "XYZ":
        monkeypatch.setenv(f"PS_PLAN_{ax}", str(pv))


def _largest_prime(n):
    f, p = 1, 2
    while p * p <= n:
        while n % p == 0:
            f, n = p, n // p
        p += 1
    return max(f, n) if n > 1 else f


# padded 194 x 40 x 34: x = 2 x 97 (96 = 2^5 3), z = 2 x 17 (16 = 2^4); y = 5 x 8
NC, BC = (97, 20, 17), (0, 0, 0)


@pytest.mark.parametrize("pv", [RADER, RADER | 1, RADER | 2, RADER | 3])
def test_rader_plan_matches_oracle_and_reports_its_stages(native, oracle, monkeypatch, pv):
    monkeypatch.setenv("PS_KERNELS", "runtime")
    _set_plan(monkeypatch, pv)
    dx = tuple(2.0 / n for n in NC)
    B = _fields(NC, 3)
    ref, _ = oracle.solve3d(NC, BC, dx, B, 2, curl=True)
    got, _ = native.solve(NC, BC, dx, B, 2, precision="fp32", curl=True)
    assert rel_l2(got, ref) < FP32_TOL
    with native.PoissonSolver() as s:
        s.setup3d(NC, BC, dx, 2)
        s.set_return_curl(True)
        s.set_precision("fp32")
        plans = s.pass_plan(7)
        assert plans[0] == ([97, 2], 96) and plans[4] == ([97, 2], 96)
        assert plans[2] == ([17, 2], 16)
        assert plans[1] == ([5, 8], 0)


# every prime factor 17 .. 97 that Rader's algorithm takes (p - 1 13-smooth),
# periodic (L = p: the Rader stage alone) and unbounded (L = 2 p) along x;
# 23, 53, 67, 79 and 89 put radix-11 or radix-13 stages in the sub-transform
PRIMES = [17, 19, 23, 29, 31, 37, 41, 43, 53, 61, 67, 71, 73, 79, 89, 97]


@pytest.mark.parametrize("n", PRIMES)
@pytest.mark.parametrize("bcx", [0, 1])
def test_rader_lengths_match_oracle(native, oracle, monkeypatch, n, bcx):
    monkeypatch.setenv("PS_KERNELS", "runtime")
    _set_plan(monkeypatch, RADER)
    nc, bc = (n, 6, 8), (bcx, bcx, 1)
    dx = tuple(2.0 / m for m in nc)
    B = _fields(nc, n + 100 * bcx, 1)
    if bc == (1, 1, 1):
        B[0] -= B[0].mean()
    ref, _ = oracle.solve3d(nc, bc, dx, B + [None, None], 2, grad=True)
    got, _ = native.solve(nc, bc, dx, B + [None, None], 2, precision="fp32", grad=True)
    assert rel_l2(got, ref) < FP32_TOL
    with native.PoissonSolver() as s:
        s.setup3d(nc, bc, dx, 2)
        s.set_return_grad(True)
        s.set_precision("fp32")
        stages, m = s.pass_plan(1)[0]
        assert stages[0] == n and m == n - 1
        assert stages == ([n] if bcx else [n, 2])


def test_non_rader_lengths_keep_bluestein(native, monkeypatch):
    """p = 47 (46 = 2 x 23) and p = 103 (102 = 6 x 17): the variant bit is
    ignored and Bluestein's algorithm runs."""
    monkeypatch.setenv("PS_KERNELS", "runtime")
    _set_plan(monkeypatch, RADER)
    for n in (47, 103):
        nc = (n, 6, 8)
        with native.PoissonSolver() as s:
            s.setup3d(nc, (1, 1, 1), tuple(2.0 / m for m in nc), 2)
            s.set_precision("fp32")
            stages, m = s.pass_plan(1)[0]
            assert m >= 2 * n - 1 and _largest_prime(m) <= 5


def test_fp64_ignores_rader_variant(native, monkeypatch):
    monkeypatch.setenv("PS_KERNELS", "runtime")
    dx = tuple(2.0 / n for n in NC)
    B = _fields(NC, 4)
    base, _ = native.solve(NC, BC, dx, B, 2, precision="fp64", curl=True)
    _set_plan(monkeypatch, RADER | 3)
    got, _ = native.solve(NC, BC, dx, B, 2, precision="fp64", curl=True)
    for a, b in zip(got, base):
        assert np.array_equal(a, b)


# a batch mixing Rader lengths (34, 74, 38, 46, 62, 82, 194), Bluestein-only
# ones (47 periodic: 46 = 2 x 23) and others, on every boundary family
BATCH = [
    ((17, 19, 23), (1, 1, 1), dict(curl=True)),
    ((37, 10, 17), (0, 0, 0), dict()),
    ((29, 29, 31), (1, 1, 0), dict(div=True)),
    ((12, 41, 19), (0, 0, 1), dict(grad=True)),
    ((97, 8, 6), (0, 0, 0), dict()),
    ((47, 9, 14), (1, 1, 1), dict(curl=True)),
    ((16, 12, 10), (0, 0, 0), dict()),
]


def _batch_fields(nc, opts, seed, zero_mean):
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


def test_rader_in_a_batch(native, oracle):
    b = native.PoissonBatch("fp32")
    data = []
    for i, (nc, bc, opts) in enumerate(BATCH):
        b.add(nc, bc, tuple(2.0 / n for n in nc), 2)
        for o in ("grad", "div", "curl"):
            if opts.get(o):
                getattr(b, f"set_return_{o}")(i, True)
        B = _batch_fields(nc, opts, 90 + i, zero_mean=bc == (1, 1, 0))
        b.push(i, *B)
        data.append(B)

    def pull_all():
        out = []
        for i, (nc, bc, opts) in enumerate(BATCH):
            shape = (nc[2], nc[1], nc[0])
            A = [np.full(shape, np.nan) for _ in range(3)]
            b.pull(i, *A)
            out.append([a if not np.isnan(a).all() else None for a in A])
        return out

    b.solve()
    blue = pull_all()
    for ax in range(3):
        b.set_tuning(ax, 256, 16, RADER)
    assert [v for _, _, v in b.tuning()] == [RADER] * 3
    b.solve()
    rad = pull_all()
    for i, (nc, bc, opts) in enumerate(BATCH):
        ref, _ = oracle.solve3d(nc, bc, tuple(2.0 / n for n in nc), data[i], 2, **opts)
        assert rel_l2(rad[i], ref) < FP32_TOL, (i, nc, bc)
        assert rel_l2(rad[i], blue[i]) < 1e-6, (i, nc, bc)
    with pytest.raises(native.PSError):
        b.set_tuning(0, 48, 16, 0)  # not a multiple of 32
    with pytest.raises(native.PSError):
        b.set_tuning(0, 256, 16, 8)  # no such variant
    b.close()
