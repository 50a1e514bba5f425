"""Plan variants of the run-time transform kernels (FP32): the power-of-two
part of a length in radix 16 or radix 8 (PS_PLAN_* bit 0), and Bluestein's
convolution length as the least power of two or the least 2^a 3^b 5^c
>= 2 L - 1 (bit 1). Each variant must give the oracle's results to FP32
tolerance; FP64 transforms ignore the variants (bit-identical results); and
ps_get_pass_plan must report the stages each variant runs.
"""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu

FP32_TOL = 5e-6


def _fields(nc, seed, ncomp=3):
    rng = np.random.default_rng(seed)
    return [rng.standard_normal((nc[2], nc[1], nc[0])) for _ in range(ncomp)]


def _next_smooth(n):
    """least 2^a 3^b 5^c >= n"""
    m = n
    while True:
        x = m
        for p in (2, 3, 5):
            while x % p == 0:
                x //= p
        if x == 1:
            return m
        m += 1


def _set_plan(monkeypatch, pv):
    for ax in "XYZ":
        monkeypatch.setenv(f"PS_PLAN_{ax}", str(pv))


# padded 194 x 40 x 34: x and z by Bluestein (97 and 17 are prime), y = 5 x 8
NC, BC = (97, 20, 17), (0, 0, 0)
# (x stages, x convolution length, z stages, z convolution length) for each variant
EXPECTED = {
    0: ([16, 16, 2], 512, [8, 8, 2], 128),
    1: ([8, 8, 8], 512, [8, 8, 2], 128),    # z holds 8 elements a thread: no radix cap below it
    2: ([5, 5, 16], 400, [3, 3, 8], 72),    # 400 = 2^4 5^2 >= 387, 72 = 2^3 3^2 >= 67
    3: ([5, 5, 8, 2], 400, [3, 3, 8], 72),
}


@pytest.mark.parametrize("pv", [0, 1, 2, 3])
def test_plan_variant_matches_oracle_and_reports_its_stages(native, oracle, monkeypatch, pv):
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
        xs, xm, zs, zm = EXPECTED[pv]
        assert plans[0] == (xs, xm) and plans[4] == (xs, xm)
        assert plans[2] == (zs, zm)
        assert plans[1] == ([5, 8], 0)  # 40: no power-of-two part above 8, no Bluestein
        # FP64 transforms take the default plan (8 elements a thread) whatever the variant
        s.set_precision("fp64")
        assert s.pass_plan(7)[0] == ([8, 8, 8], 512)


def test_fp64_ignores_plan_variants(native, monkeypatch):
    monkeypatch.setenv("PS_KERNELS", "runtime")
    dx = tuple(2.0 / n for n in NC)
    B = _fields(NC, 4)
    base, _ = native.solve(NC, BC, dx, B, 2, precision="fp64", curl=True)
    _set_plan(monkeypatch, 3)
    got, _ = native.solve(NC, BC, dx, B, 2, precision="fp64", curl=True)
    for a, b in zip(got, base):
        assert np.array_equal(a, b)


# Bluestein on a smooth convolution length for prime factors 17 .. 97, periodic
# (L = n) and unbounded (L = 2 n) along x
PRIMES = [17, 19, 23, 29, 31, 37, 41, 43, 47, 53, 59, 61, 67, 71, 73, 79, 83, 89, 97]


@pytest.mark.parametrize("n", PRIMES)
@pytest.mark.parametrize("bcx", [0, 1])
def test_smooth_bluestein_lengths_match_oracle(native, oracle, monkeypatch, n, bcx):
    monkeypatch.setenv("PS_KERNELS", "runtime")
    _set_plan(monkeypatch, 2)
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
        L = n if bcx else 2 * n
        assert m == _next_smooth(2 * L - 1) <= 1 << (2 * L - 2).bit_length()
        assert all(r in (2, 3, 4, 5, 8, 16) for r in stages)
        assert int(np.prod(stages)) == m


def test_autotune_considers_plan_variants(native, tmp_path, monkeypatch):
    """Tuning an FP32 configuration with Bluestein lengths keeps the results
    within FP32 rounding of the default plan and reports a valid plan."""
    monkeypatch.setenv("PS_TUNE_CACHE", str(tmp_path / "tune.txt"))
    dx = tuple(2.0 / n for n in NC)
    B = _fields(NC, 5)
    with native.PoissonSolver() as s:
        s.setup3d(NC, BC, dx, 2)
        s.set_return_curl(True)
        s.set_precision("fp32")
        s.push(*B)
        s.solve3d()
        shape = (NC[2], NC[1], NC[0])
        A0 = [np.empty(shape) for _ in range(3)]
        s.pull(*A0)
        s.autotune(7)
        s.solve3d()
        A1 = [np.empty(shape) for _ in range(3)]
        s.pull(*A1)
        assert rel_l2(A1, A0) < 1e-6
        xs, xm = s.pass_plan(7)[0]
        assert (xs, xm) in [EXPECTED[v][:2] for v in range(4)] + [([97, 2], 96)]  # or Rader's (bit 2)
    lines = (tmp_path / "tune.txt").read_text().split("\n")
    assert all(0 <= int(l.split()[3]) <= 7 for l in lines if l)
