"""Every FP32 z-pass kernel family against the oracle, at the z lengths the
wide kernels cover (Pz = 256 .. 2048), for every spectral operation.

The families: the warp-per-column kernel fed by tiled bulk copies
(PS_KERNELS_Z=tma, the default on unbounded z of 256..1024 points), the
kernel with its DFT stages on the tensor cores (PS_KERNELS_Z=tc: unbounded z
of 1024 points, the (4, 6, 512) shape here), the
tensor-memory fused kernel (PS_KERNELS_Z=tmem, the default elsewhere), the
shared-memory fused kernel (PS_KERNELS_Z=wide) and the length-specialised
one (PS_KERNELS_Z=p2). A family that does not cover a shape falls back to
the default. Narrow x-y extents keep the oracle fast while the z
columns reach the long lengths; the narrow x extent also leaves part of each
CTA's columns inactive.
"""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu

FP32_TOL = 5e-6

# (ncell, bc) -> Pz: 256, 512, 1024, 2048 unbounded; 1024 and 512 periodic in z
SHAPES = [
    ((6, 5, 128), (0, 0, 0)),
    ((5, 6, 256), (0, 0, 0)),
    ((4, 6, 512), (0, 0, 0)),
    ((4, 4, 1024), (0, 0, 0)),
    ((6, 4, 1024), (1, 1, 1)),
    ((8, 6, 512), (0, 0, 1)),
]

# (options, components pushed)
OPS = [
    (dict(), (0, 1, 2)),
    (dict(), (1,)),
    (dict(grad=True), (0,)),
    (dict(grad=True), (0, 1, 2)),
    (dict(div=True), (0, 1, 2)),
    (dict(curl=True), (0, 1, 2)),
]

FAMILIES = ["tmem", "wide", "p2", "tma", "tc"]


def _fields(nc, comps, seed):
    rng = np.random.default_rng(seed)
    shape = (nc[2], nc[1], nc[0])
    return [rng.standard_normal(shape) if c in comps else None for c in range(3)]


_ref_cache = {}


def _reference(oracle, si, oi):
    key = (si, oi)
    if key not in _ref_cache:
        nc, bc = SHAPES[si]
        opts, comps = OPS[oi]
        dx = (2.0 / nc[0], 1.5 / nc[1], 2.5 / nc[2])
        B = _fields(nc, comps, 10 * si + oi)
        ref, _ = oracle.solve3d(nc, bc, dx, B, 2, **opts)
        _ref_cache[key] = (dx, B, ref)
    return _ref_cache[key]


@pytest.mark.parametrize("family", FAMILIES)
@pytest.mark.parametrize("oi", range(len(OPS)))
@pytest.mark.parametrize("si", range(len(SHAPES)))
def test_fp32_z_family_vs_oracle(native, oracle, monkeypatch, si, oi, family):
    nc, bc = SHAPES[si]
    opts, _ = OPS[oi]
    dx, B, ref = _reference(oracle, si, oi)
    monkeypatch.setenv("PS_KERNELS_Z", family)
    got, _ = native.solve(nc, bc, dx, B, 2, precision="fp32", **opts)
    assert rel_l2(got, ref) < FP32_TOL


@pytest.mark.parametrize("lines", [1, 2, 4, 8])
def test_tmem_z_lines_per_cta(native, oracle, monkeypatch, lines):
    """The tensor-memory kernel with 1..8 columns a CTA at Pz = 1024 (1..8 warps)."""
    si, oi = 2, 5
    nc, bc = SHAPES[si]
    opts, _ = OPS[oi]
    dx, B, ref = _reference(oracle, si, oi)
    monkeypatch.setenv("PS_KERNELS_Z", "tmem")
    monkeypatch.setenv("PS_LINES_Z", str(lines))
    got, _ = native.solve(nc, bc, dx, B, 2, precision="fp32", **opts)
    assert rel_l2(got, ref) < FP32_TOL


# tall y extents: the wide y kernels at P_y = 256 .. 1024, unbounded (the
# zero-padded half pruned) and periodic, and the bulk-copy y kernels
# (PS_KERNELS_Y=tma: unbounded only, the periodic shapes fall back)
Y_SHAPES = [
    ((6, 128, 8), (0, 0, 0)),
    ((4, 256, 6), (0, 0, 0)),
    ((4, 512, 4), (0, 0, 0)),
    ((6, 256, 6), (1, 1, 1)),
    ((5, 512, 7), (0, 0, 1)),
]


@pytest.mark.parametrize("family", ["wide", "tma"])
@pytest.mark.parametrize("yi", range(len(Y_SHAPES)))
def test_fp32_y_family_vs_oracle(native, oracle, monkeypatch, yi, family):
    nc, bc = Y_SHAPES[yi]
    monkeypatch.setenv("PS_KERNELS_Y", family)
    dx = (2.0 / nc[0], 1.5 / nc[1], 2.5 / nc[2])
    B = _fields(nc, (0, 1, 2), 500 + yi)
    ref, _ = oracle.solve3d(nc, bc, dx, B, 2, curl=True)
    got, _ = native.solve(nc, bc, dx, B, 2, precision="fp32", curl=True)
    assert rel_l2(got, ref) < FP32_TOL


# long x extents: the length-specialised x kernels (PS_KERNELS_X=p2) and the
# warp-per-line x kernels (PS_KERNELS_X=tma) at P_x = 256 .. 1024, unbounded
# (the zero-padded half pruned) and periodic; odd row counts leave a lone
# last row
X_SHAPES = [
    ((128, 6, 8), (0, 0, 0)),
    ((256, 5, 4), (0, 0, 0)),
    ((512, 4, 4), (0, 0, 0)),
    ((256, 6, 6), (1, 1, 1)),
    ((512, 3, 5), (1, 1, 0)),
]


@pytest.mark.parametrize("family", ["p2", "tma"])
@pytest.mark.parametrize("xi", range(len(X_SHAPES)))
def test_fp32_x_family_vs_oracle(native, oracle, monkeypatch, xi, family):
    nc, bc = X_SHAPES[xi]
    monkeypatch.setenv("PS_KERNELS_X", family)
    dx = (2.0 / nc[0], 1.5 / nc[1], 2.5 / nc[2])
    rng = np.random.default_rng(600 + xi)
    B = [rng.standard_normal((nc[2], nc[1], nc[0])) for _ in range(3)]
    if bc == (1, 1, 0):
        B = [b - b.mean(axis=(1, 2), keepdims=True) for b in B]
    ref, _ = oracle.solve3d(nc, bc, dx, B, 2, curl=True)
    got, _ = native.solve(nc, bc, dx, B, 2, precision="fp32", curl=True)
    # Periodic x of 512 points with a 3-cell y: the solution lives in the few
    # lowest k_x modes (1/k^2 up to (N/2)^2 = 65536 times the highest), while
    # white noise puts the FP32 rounding of the transforms (about eps |B|) into
    # those modes too, so the relative error is larger (1.9e-5 measured).
    tol = 5e-5 if nc == (512, 3, 5) else FP32_TOL
    assert rel_l2(got, ref) < tol
