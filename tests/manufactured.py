"""Manufactured solutions of the reference's four 3D validation programs
(c++/test/{unbounded3d,periodic3d,mixed_ppf3d,mixed_ffp3d}/sources/main.cpp),
restated in numpy: the source B, the analytic output, and the relative L2
error each program prints ("Error: dx rel_L2"), computed the same way
(cell-centred points, sum over the three components).

The printed errors of the reference, run single-rank in this project's
oracle build, are the known answers the tests pin against.
"""
from __future__ import annotations

import numpy as np

PI = np.pi
C = 10.0

KNOWN_ERRORS = {
    "unbounded3d": 2.797557e-10,
    "periodic3d": 9.528272e-16,
    "mixed_ppf3d": 2.012790e-10,
    "mixed_ffp3d": 3.071677e-10,
}

SETUPS = {
    # name: (xmin, xmax, ncell, bc, option)
    "unbounded3d": ((-0.5, -1.0, -1.0), (0.5, 1.0, 1.0), (64, 128, 128), (0, 0, 0), "curl"),
    "periodic3d": ((-1.0, -1.0, -1.0), (1.0, 1.0, 1.0), (64, 64, 64), (1, 1, 1), "curl"),
    "mixed_ppf3d": ((-1.0, -1.0, -1.0), (1.0, 1.0, 1.0), (64, 64, 64), (1, 1, 0), "curl"),
    "mixed_ffp3d": ((-1.0, -1.0, -1.0), (1.0, 1.0, 1.0), (64, 64, 64), (0, 0, 1), "grad"),
}


def grid(name, ncell=None):
    xmin, xmax, nc, bc, opt = SETUPS[name]
    nc = ncell or nc
    dx = tuple((xmax[d] - xmin[d]) / nc[d] for d in range(3))
    x = xmin[0] + (np.arange(nc[0]) + 0.5) * dx[0]
    y = xmin[1] + (np.arange(nc[1]) + 0.5) * dx[1]
    z = xmin[2] + (np.arange(nc[2]) + 0.5) * dx[2]
    Z, Y, X = np.meshgrid(z, y, x, indexing="ij")
    return nc, bc, dx, opt, X, Y, Z


def unbounded3d(X, Y, Z):
    """Compact vortex ring (c = 10, r0 = 0.5), axis along x; curl of A."""
    r0 = 0.5
    rho = np.sqrt(Z * Z + Y * Y)
    phi = np.sqrt((rho - r0) ** 2 + X ** 2)
    th = np.arctan2(Z, Y)
    inside = phi < r0
    q = np.where(inside, 2.0 * r0 * rho - rho ** 2 - X ** 2, 1.0)
    rr = np.where(inside, rho, 1.0)
    e = np.where(inside, np.exp(-C * r0 ** 2 / q), 0.0)
    x = X
    bmag = -e * (4 * C ** 2 * r0 ** 4 * x ** 2 * rr ** 2 - 16 * r0 ** 4 * rr ** 4 + 32 * r0 ** 3 * rr ** 5
                 - 24 * r0 ** 2 * rr ** 6 + 8 * r0 * rr ** 7 - 4 * rr ** 6 * x ** 2 - 6 * rr ** 4 * x ** 4
                 - 4 * rr ** 2 * x ** 6 - 8 * C * r0 ** 5 * rr ** 3 + 8 * C * r0 ** 4 * rr ** 4
                 - 6 * C * r0 ** 3 * rr ** 5 + 4 * C ** 2 * r0 ** 6 * rr ** 2 - 8 * C ** 2 * r0 ** 5 * rr ** 3
                 + 4 * C ** 2 * r0 ** 4 * rr ** 4 + 2 * C * r0 ** 2 * rr ** 6 + 32 * r0 ** 3 * rr ** 3 * x ** 2
                 - 48 * r0 ** 2 * rr ** 4 * x ** 2 - 24 * r0 ** 2 * rr ** 2 * x ** 4 + 24 * r0 * rr ** 5 * x ** 2
                 + 24 * r0 * rr ** 3 * x ** 4 + 8 * r0 * rr * x ** 6 + 2 * C * r0 ** 3 * rr * x ** 4
                 + 2 * C * r0 ** 2 * rr ** 2 * x ** 4 - 4 * C * r0 ** 3 * rr ** 3 * x ** 2
                 + 4 * C * r0 ** 2 * rr ** 4 * x ** 2 - rr ** 8 - x ** 8) * q ** -4 * rr ** -2
    bmag = np.where(inside, bmag, 0.0)
    B = [np.zeros_like(X), -np.sin(th) * bmag, np.cos(th) * bmag]
    amag = np.where(inside, 2.0 * C * r0 ** 2 * x * e * q ** -2, 0.0)
    solx = e * (4 * r0 ** 2 * rr ** 2 - 4 * r0 * rr ** 3 - 4 * r0 * rr * x ** 2 + rr ** 4 + 2 * rr ** 2 * x ** 2
                + x ** 4 + 2 * C * r0 ** 3 * rr - 2 * C * r0 ** 2 * rr ** 2) * q ** -2 * rr ** -1
    solx = np.where(inside, solx, 0.0)
    sol = [solx, np.cos(th) * amag, np.sin(th) * amag]
    return B, sol


def periodic3d(X, Y, Z):
    s, c = np.sin, np.cos
    t = 2.0 * PI
    B = [-s(t * X) * c(t * Y) * s(t * Z), -c(t * X) * s(t * Y) * s(t * Z), -2.0 * c(t * X) * c(t * Y) * c(t * Z)]
    sol = [c(t * X) * s(t * Y) * c(t * Z) / t, -s(t * X) * c(t * Y) * c(t * Z) / t, np.zeros_like(X)]
    return B, sol


def mixed_ppf3d(X, Y, Z):
    inside = np.abs(Z) < 1.0
    zz = np.where(inside, Z, 0.0)
    den = (zz - 1.0) * (zz + 1.0)
    e = np.where(inside, np.exp(C * zz ** 2 / den), 0.0)
    bx = e * np.sin(PI * X) * np.sin(PI * Y) * (
        2 * PI ** 2 * zz ** 8 - 8 * PI ** 2 * zz ** 6 + 12 * PI ** 2 * zz ** 4 - 6 * C * zz ** 4
        - 8 * PI ** 2 * zz ** 2 - 4 * C ** 2 * zz ** 2 + 4 * C * zz ** 2 + 2 * PI ** 2 + 2 * C) / ((zz - 1.0) ** 4 * (zz + 1.0) ** 4)
    B = [np.where(inside, bx, 0.0), np.zeros_like(X), np.zeros_like(X)]
    soly = -2.0 * C * zz * e * np.sin(PI * X) * np.sin(PI * Y) / ((zz - 1.0) ** 2 * (zz + 1.0) ** 2)
    solz = -PI * e * np.sin(PI * X) * np.cos(PI * Y)
    sol = [np.zeros_like(X), np.where(inside, soly, 0.0), np.where(inside, solz, 0.0)]
    return B, sol


def mixed_ffp3d(X, Y, Z, dx0):
    r0 = 1.0
    r = np.sqrt(X * X + Y * Y)
    inside = r < r0
    q = np.where(inside, r0 ** 2 - X ** 2 - Y ** 2, 1.0)
    e = np.where(inside, np.exp(-C * r0 ** 2 / q), 0.0)
    bx = 4.0 * C * r0 ** 2 * e * (r0 ** 4 - X ** 4 - Y ** 4 - 2 * X ** 2 * Y ** 2 - C * X ** 2 * r0 ** 2
                                  - C * Y ** 2 * r0 ** 2) * q ** -4
    bx = np.where(inside, bx, 0.0)
    B = [bx, bx.copy(), bx.copy()]
    keep = inside & ~(r < 0.25 * dx0)
    solx = np.where(keep, -2.0 * C * r0 ** 2 * X * e * q ** -2, 0.0)
    soly = np.where(keep, -2.0 * C * r0 ** 2 * Y * e * q ** -2, 0.0)
    sol = [solx, soly, np.zeros_like(X)]
    return B, sol


def case(name, ncell=None):
    nc, bc, dx, opt, X, Y, Z = grid(name, ncell)
    if name == "unbounded3d":
        B, sol = unbounded3d(X, Y, Z)
    elif name == "periodic3d":
        B, sol = periodic3d(X, Y, Z)
    elif name == "mixed_ppf3d":
        B, sol = mixed_ppf3d(X, Y, Z)
    else:
        B, sol = mixed_ffp3d(X, Y, Z, dx[0])
    return nc, bc, dx, opt, B, sol


def printed_error(A, sol, dx):
    """The rel-L2 error the reference programs print (cell volume weights cancel)."""
    dv = dx[0] * dx[1] * dx[2]
    err = sum(float(np.sum(dv * (a - s) ** 2)) for a, s in zip(A, sol))
    nrm = sum(float(np.sum(dv * s ** 2)) for s in sol)
    return (err / nrm) ** 0.5
