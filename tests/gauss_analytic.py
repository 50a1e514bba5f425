"""Closed-form and quadrature solutions for the Gaussian-regularised kernel
family (order 2m, width sig): its spectrum is zeta_m(sig|k|)/|k|^2 with
zeta_m(k) = e^{-a} sum_{n<m} a^n/n!, a = sig^2 k^2/2.

For a unit Gaussian source of width s, each term e^{-a} a^n/n! times the
source spectrum e^{-s^2 k^2/2} equals (sig/S)^{2n} times the same term at
width S = sqrt(sig^2 + s^2), so the free-space solution is
sum_n (sig/S)^{2n} G_n^{(S)}, with G_n the family's terms (G_0 the Gaussian
potential). Modes with a periodic wavenumber kappa along the unbounded
axes are one-dimensional quadratures of the spectrum. Used by the oracle
tests and the GPU tests alike.
"""
import numpy as np
from scipy import integrate, special

L_BOX = 2.0  # every case lives on [-1, 1] per axis


def zeta(k, m, sig):
    a = 0.5 * (sig * np.asarray(k, dtype=float)) ** 2
    return np.exp(-a) * sum(a ** n / special.factorial(n) for n in range(m))


def composed(green, d, m, sig, s, r):
    """Solution for a unit Gaussian source of width s; green(d, m, S, r) is
    the family's kernel (oracle.gauss_green)."""
    S = np.sqrt(sig * sig + s * s)

    def one(rr):
        v = green(d, 1, S, rr)
        for n in range(1, m):
            v += (sig / S) ** (2 * n) * (green(d, n + 1, S, rr) - green(d, n, S, rr))
        return v

    r = np.asarray(r, dtype=float)
    flat = np.array([one(x) for x in r.ravel()])
    return flat.reshape(r.shape)


def cell_centres(n):
    h = L_BOX / n
    return -L_BOX / 2 + (np.arange(n) + 0.5) * h, h


def line_profile(z, kappa, m, sig, s):
    """(1/pi) int_0^inf zeta(sqrt(kappa^2+k^2)) e^{-s^2k^2/2} cos(kz) / (kappa^2+k^2) dk:
    the response along an unbounded axis to a Gaussian profile times a
    periodic mode of wavenumber kappa."""
    f = lambda k, zz: zeta(np.hypot(kappa, k), m, sig) * np.exp(-0.5 * (s * k) ** 2) * np.cos(k * zz) / (kappa ** 2 + k ** 2)
    return np.array([integrate.quad(f, 0, 80 / s, args=(zz,), limit=4000, epsabs=1e-15)[0] / np.pi for zz in z])


def plane_profile(rho, q, m, sig, s):
    """(1/2pi) int_0^inf zeta(sqrt(k^2+q^2)) e^{-s^2k^2/2} J0(k rho) k / (k^2+q^2) dk:
    the response in an unbounded plane to a 2D Gaussian times a periodic
    mode of wavenumber q normal to it."""
    f = lambda k, r: zeta(np.hypot(k, q), m, sig) * np.exp(-0.5 * (s * k) ** 2) * special.j0(k * r) * k / (k ** 2 + q ** 2)
    rs, inv = np.unique(np.round(np.asarray(rho, dtype=float), 13), return_inverse=True)
    vals = np.array([integrate.quad(f, 0, 80 / s, args=(r,), limit=4000, epsabs=1e-15)[0] / (2 * np.pi) for r in rs])
    return vals[inv].reshape(np.shape(rho))


def case3d(green, bc, n, m, s=0.12, kk=4):
    """(B, A_exact, RB_exact or None) on n^3 cells of [-1, 1]^3 with the
    default width 2h."""
    x, h = cell_centres(n)
    sig = 2 * h
    Z, Y, X = np.meshgrid(x, x, x, indexing="ij")
    if bc == (0, 0, 0):
        R = np.sqrt(X ** 2 + Y ** 2 + Z ** 2)
        B = np.exp(-R ** 2 / (2 * s * s)) / (2 * np.pi * s * s) ** 1.5
        return B, composed(green, 3, m, sig, s, R), None
    if bc == (1, 1, 0):
        g1 = np.exp(-Z ** 2 / (2 * s * s)) / np.sqrt(2 * np.pi * s * s)
        mode = np.cos(2 * np.pi * kk * X / L_BOX) * np.cos(2 * np.pi * kk * Y / L_BOX)
        kap = 2 * np.pi * np.hypot(kk, kk) / L_BOX
        ex = composed(green, 1, m, sig, s, Z) + mode * line_profile(x, kap, m, sig, s)[:, None, None]
        return g1 * (1.0 + mode), ex, None
    if bc == (0, 0, 1):
        Rr = np.hypot(X, Y)
        g2 = np.exp(-Rr ** 2 / (2 * s * s)) / (2 * np.pi * s * s)
        mode = np.cos(2 * np.pi * kk * Z / L_BOX)
        q = 2 * np.pi * kk / L_BOX
        rr = np.hypot(*np.meshgrid(x, x, indexing="ij"))
        ex = composed(green, 2, m, sig, s, Rr) + mode * plane_profile(rr, q, m, sig, s)[None, :, :]
        return g2 * (1.0 + mode), ex, None
    modes = [(1, 2, 3, 0.7), (5, 0, 1, -1.3), (2, 7, 4, 0.4)]
    B = np.zeros_like(X)
    A = np.zeros_like(X)
    RB = np.zeros_like(X)
    for i, j, k, a in modes:
        c = np.cos(2 * np.pi * (i * X + j * Y + k * Z) / L_BOX)
        kn = 2 * np.pi * np.sqrt(i * i + j * j + k * k) / L_BOX
        B += a * c
        A += a * zeta(kn, m, sig) / kn ** 2 * c
        RB += a * zeta(kn, m, sig) * c
    return B, A, RB


def case2d(green, bc, n, m, s=0.12, kk=4):
    """(B, A_exact) on n^2 cells of [-1, 1]^2, fields [Ny][Nx]."""
    x, h = cell_centres(n)
    sig = 2 * h
    Y, X = np.meshgrid(x, x, indexing="ij")
    if bc == (0, 0):
        R = np.hypot(X, Y)
        B = np.exp(-R ** 2 / (2 * s * s)) / (2 * np.pi * s * s)
        return B, composed(green, 2, m, sig, s, R)
    if bc == (1, 1):
        B = np.zeros_like(X)
        A = np.zeros_like(X)
        for i, j, a in [(1, 2, 0.7), (5, 1, -1.3)]:
            c = np.cos(2 * np.pi * (i * X + j * Y) / L_BOX)
            kn = 2 * np.pi * np.hypot(i, j) / L_BOX
            B += a * c
            A += a * zeta(kn, m, sig) / kn ** 2 * c
        return B, A
    # one unbounded axis U, one periodic axis with a mode of wavenumber kap
    U, Pd = (X, Y) if bc == (0, 1) else (Y, X)
    g1 = np.exp(-U ** 2 / (2 * s * s)) / np.sqrt(2 * np.pi * s * s)
    mode = np.cos(2 * np.pi * kk * Pd / L_BOX)
    kap = 2 * np.pi * kk / L_BOX
    prof = line_profile(x, kap, m, sig, s)
    F = prof[None, :] if bc == (0, 1) else prof[:, None]
    return g1 * (1.0 + mode), composed(green, 1, m, sig, s, U) + mode * F
