"""Double-float transforms (PS_PREC_DF64): FP64 kernel build, FFT stages and
spectral operation in pairs of FP32 numbers (about 48 significant bits),
FP64 field input and output. Against the oracle (the reference's FP64
algorithm) at FP64-class tolerance on every boundary family, operation and
transform kind (power-of-two, mixed-radix, direct prime stages, Bluestein),
the 2D solver and the returned right-hand side; and the option's plumbing.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

DF_L2 = 1e-12   # relative L2 against the oracle
DF_MAX = 1e-11  # max |A - A_ref| / max |A_ref|


def _errors(got, ref):
    num = den = dmax = rmax = 0.0
    for g, r in zip(got, ref):
        if r is None:
            continue
        d = np.asarray(g) - r
        num += float(np.sum(d * d))
        den += float(np.sum(r * r))
        dmax = max(dmax, float(np.abs(d).max()))
        rmax = max(rmax, float(np.abs(r).max()))
    return (num / den) ** 0.5, dmax / rmax


def _fields(nc, comps, seed, zero_mean=False):
    rng = np.random.default_rng(seed)
    B = [rng.standard_normal((nc[2], nc[1], nc[0])) if c in comps else None for c in range(3)]
    if zero_mean:
        B = [b - b.mean(axis=(1, 2), keepdims=True) if b is not None else None for b in B]
    return B


CASES = [
    # (ncell, bc, reg, options, components)
    ((24, 20, 16), (0, 0, 0), 2, dict(curl=True), (0, 1, 2)),      # powers of two
    ((18, 14, 22), (1, 1, 0), 6, dict(grad=True), (0,)),           # mixed radix (3, 7, 11)
    ((16, 12, 10), (0, 0, 1), 4, dict(), (0, 1)),                  # operator none
    ((17, 12, 10), (0, 0, 0), 2, dict(curl=True), (0, 1, 2)),      # Bluestein (34 = 2 x 17)
    ((20, 16, 12), (1, 1, 1), 10, dict(div=True), (0, 1, 2)),      # fully periodic, div
    ((26, 22, 13), (1, 1, 0), 0, dict(curl=True), (0, 1, 2)),      # direct radix 11 and 13 stages
]


@pytest.mark.parametrize("case", CASES)
def test_df64_matches_oracle(native, oracle, case):
    nc, bc, reg, opts, comps = case
    dx = (2.0 / nc[0], 1.5 / nc[1], 2.5 / nc[2])
    B = _fields(nc, comps, sum(nc) + reg, zero_mean=bc != (0, 0, 0))
    ref, _ = oracle.solve3d(nc, bc, dx, B, reg, **opts)
    got, _ = native.solve(nc, bc, dx, B, reg, precision="df64", **opts)
    l2, mx = _errors(got, ref)
    print(f"{nc} {bc} {opts}: rel L2 {l2:.2e}, max {mx:.2e}")
    assert l2 < DF_L2 and mx < DF_MAX


def test_df64_returned_rhs_and_reprojection(native, oracle):
    nc, bc, reg = (20, 18, 16), (0, 0, 0), 4
    dx = tuple(2.0 / n for n in nc)
    B = _fields(nc, (0, 1, 2), 71)
    ref, rb_ref = oracle.solve3d(nc, bc, dx, B, reg, curl=True, reproject=True, want_rhs=True)
    got, rb = native.solve(nc, bc, dx, B, reg, precision="df64", curl=True, reproject=True, want_rhs=True)
    assert _errors(got, ref)[0] < DF_L2
    assert _errors(rb, rb_ref)[0] < DF_L2


def test_df64_2d(native, oracle):
    import ctypes

    from poisson_solver_gb300 import _lib as L
    nc, bc = (40, 36), (0, 0)
    dx = (2.0 / 40, 2.0 / 36)
    rng = np.random.default_rng(5)
    B = rng.standard_normal((nc[1], nc[0]))
    ref, _ = oracle.solve2d(nc, bc, dx, [B, None, None], 2, grad=True)
    with native.PoissonSolver() as s:
        s.setup2d(nc, bc, dx, 2)
        s.set_return_grad(True)
        s.set_precision("df64")
        v = ctypes.c_int()
        assert s._lib.ps_get_option(s._h, L.PS_OPT_PRECISION, ctypes.byref(v)) == 0 and v.value == L.PS_PREC_DF64
        s.push(B)
        s.solve2d()
        A = [np.empty_like(B) for _ in range(3)]
        s.pull(*A)
    assert _errors(A, ref)[0] < DF_L2


def test_df64_ring_source_128(native, oracle):
    """The benchmark's 16-ring source sampled at 128^3 (reg 10, curl)."""
    import bench
    w = dict(bench.WORKLOADS["rings512"], n=128)
    B = [b.numpy() for b in bench.make_source(w, "cpu")]
    nc, dx = (128,) * 3, (2.0 / 128,) * 3
    ref, _ = oracle.solve3d(nc, (0, 0, 0), dx, B, reg=10, curl=True)
    got, _ = native.solve(nc, (0, 0, 0), dx, B, 10, precision="df64", curl=True)
    l2, mx = _errors(got, ref)
    print(f"rings 128^3 df64: rel L2 {l2:.2e}, max {mx:.2e}")
    assert l2 < DF_L2 and mx < DF_MAX


def test_df64_runs_on_the_runtime_kernels(native):
    with native.PoissonSolver() as s:
        s.setup3d((128, 128, 128), (0, 0, 0), (2.0 / 128,) * 3, 2)
        s.set_return_curl(True)
        s.set_precision("df64")
        assert all(f == "runtime" for f, _ in s.pass_config(7))


def test_batch_rejects_df64(native):
    from poisson_solver_gb300 import PSError
    from poisson_solver_gb300 import _lib as L
    with pytest.raises(PSError) as e:
        native.PoissonBatch("df64")
    assert e.value.status == L.PS_ERR_UNSUPPORTED
