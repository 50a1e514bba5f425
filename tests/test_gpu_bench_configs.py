"""The benchmarked configurations against the oracle, at sizes the oracle runs
in seconds:

* the 64^3 unbounded scalar Gaussian (sigma 0.1 at the origin), reg 2 --
  the reference's own CPU-runnable case, at its stated size;
* the perturbed vortex ring of the 256^3 vector case (reg 6, curl) at 128^3;
* the mixed periodic-periodic-unbounded Fourier-mode source of the
  512x512x256 case (grad of the scalar pushed in 3 components, div of
  (B, B, B)) at 128x128x64;
* the 16-ring source of the 512^3 headline case (reg 10, curl) at 128^3;
* the bulk-copy (tile-queue) kernels at transform length 1024 along each
  axis in turn, with many tiles per persistent CTA: 64x64x512, 64x512x64 and
  512x64x64 unbounded curl solves (padded 128x128x1024 and its turns).

Every case states relative L2 and maximum error (max |A - A_ref| over
max |A_ref|) against the oracle, FP64 and FP32 transforms.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FP64_L2, FP64_MAX = 1e-12, 1e-11
FP32_L2, FP32_MAX = 5e-6, 5e-5


def errors(got, ref):
    num = den = 0.0
    dmax = rmax = 0.0
    for g, r in zip(got, ref):
        if r is None:
            assert g is None
            continue
        d = np.asarray(g) - r
        num += float(np.sum(d * d))
        den += float(np.sum(r * r))
        dmax = max(dmax, float(np.abs(d).max()))
        rmax = max(rmax, float(np.abs(r).max()))
    return (num / den) ** 0.5, dmax / rmax


def check(native, nc, bc, dx, B, ref, reg, precisions=("fp64", "fp32"), **opts):
    out = {}
    for prec in precisions:
        got, _ = native.solve(nc, bc, dx, B, reg, precision=prec, **opts)
        l2, mx = errors(got, ref)
        print(f"{nc} {bc} {opts} {prec}: rel L2 {l2:.3e}, max {mx:.3e}")
        if prec == "fp64":
            assert l2 < FP64_L2 and mx < FP64_MAX, (l2, mx)
        else:
            assert l2 < FP32_L2 and mx < FP32_MAX, (l2, mx)
        out[prec] = (l2, mx)
    return out


def test_unbounded_scalar_gaussian_64_reg2(native, oracle):
    n, s = 64, 0.1
    dx = 2.0 / n
    x = -1.0 + (np.arange(n) + 0.5) * dx
    Z, Y, X = np.meshgrid(x, x, x, indexing="ij")
    B = (2 * np.pi * s * s) ** -1.5 * np.exp(-(X * X + Y * Y + Z * Z) / (2 * s * s))
    ref, _ = oracle.solve3d((n, n, n), (0, 0, 0), (dx,) * 3, [B, None, None], reg=2)
    check(native, (n, n, n), (0, 0, 0), (dx,) * 3, [B, None, None], ref, 2)


def test_perturbed_ring_128_reg6_curl(native, oracle):
    import bench
    w = dict(bench.WORKLOADS["rings256"], n=128)
    B = [b.numpy() for b in bench.make_source(w, "cpu")]
    nc, dx = (128,) * 3, (2.0 / 128,) * 3
    ref, _ = oracle.solve3d(nc, (0, 0, 0), dx, B, reg=6, curl=True)
    check(native, nc, (0, 0, 0), dx, B, ref, 6, curl=True)


def test_sixteen_rings_128_reg10_curl(native, oracle):
    import bench
    w = dict(bench.WORKLOADS["rings512"], n=128)
    B = [b.numpy() for b in bench.make_source(w, "cpu")]
    nc, dx = (128,) * 3, (2.0 / 128,) * 3
    ref, _ = oracle.solve3d(nc, (0, 0, 0), dx, B, reg=10, curl=True)
    check(native, nc, (0, 0, 0), dx, B, ref, 10, curl=True)


@pytest.mark.parametrize("op", ["grad", "div"])
def test_mixed_fourier_modes_128x128x64(native, oracle, op):
    import bench
    w = dict(bench.WORKLOADS["mixed512"], n=(128, 128, 64))
    Bs, dx = bench.mixed_source(w, "cpu")
    Bs = Bs.numpy()
    B = [Bs, Bs, Bs]
    nc, bc = (128, 128, 64), (1, 1, 0)
    ref, _ = oracle.solve3d(nc, bc, dx, B, reg=w["reg"], **{op: True})
    check(native, nc, bc, dx, B, ref, w["reg"], **{op: True})


@pytest.mark.parametrize("nc,zfam", [((64, 64, 512), "tma"), ((64, 512, 64), "tma"), ((512, 64, 64), "tma"),
                                     ((64, 64, 512), "tc")])
def test_tile_queue_kernels_length_1024_many_tiles(native, oracle, monkeypatch, nc, zfam):
    """Transform length 1024 along one axis with the bulk-copy kernels on
    every pass (and the tensor-core z kernel): each persistent CTA takes
    several tiles, so the staging buffers' phase wrap and the tile order are
    exercised."""
    monkeypatch.setenv("PS_KERNELS", "tma")
    monkeypatch.setenv("PS_KERNELS_Z", zfam)
    rng = np.random.default_rng(sum(nc))
    B = [rng.standard_normal((nc[2], nc[1], nc[0])) for _ in range(3)]
    dx = (2.0 / nc[0], 2.0 / nc[1], 2.0 / nc[2])
    ref, _ = oracle.solve3d(nc, (0, 0, 0), dx, B, reg=2, curl=True)
    check(native, nc, (0, 0, 0), dx, B, ref, 2, precisions=("fp32",), curl=True)
    with native.PoissonSolver() as s:
        s.setup3d(nc, (0, 0, 0), dx, 2)
        s.set_return_curl(True)
        s.set_precision("fp32")
        s.push(*B)
        s.solve3d()
        fams = s.pass_config(7)
    axis = int(np.argmax(nc))
    passes = {0: (0, 4), 1: (1, 3), 2: (2,)}[axis]
    for p in passes:
        assert fams[p][0] == (zfam if p == 2 else "tma"), fams
