"""ctypes front end for the CPU oracle. TEST INFRASTRUCTURE ONLY.

Two libraries sit behind the same calls:

* ``port``      -- oracle/_build/libps_oracle.so, the plain-C restatement of the
                   reference solve (oracle/ps_oracle.c). Built anywhere.
* ``reference`` -- oracle/_ref/libpsref.so, the unmodified reference C++ sources
                   compiled with a single-rank MPI stand-in (oracle/Makefile).
                   Only buildable where the reference sources are present.

Only tests, the smoke check and the benchmark's CPU-baseline leg import this
module; the product package never does.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_SO = os.path.join(HERE, "_build", "libps_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libpsref.so")
REF_SOURCE_LINK = os.path.join(HERE, "_ref", "source")  # written by the reference build

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)
_libs: dict[str, ctypes.CDLL] = {}


def build(reference_root: str | None = None) -> None:
    """Compile the port (always) and the reference library (when reference_root,
    or else $PS_REFERENCE_ROOT, names a reference checkout that exists)."""
    ref = reference_root or os.environ.get("PS_REFERENCE_ROOT", "")
    cmd = ["make", "-s", "-f", os.path.join(HERE, "Makefile")]
    if ref and os.path.isdir(ref):
        cmd.append(f"REF={ref}")
    subprocess.run(cmd + ["all"], check=True, cwd=HERE)


def reference_root() -> str | None:
    """The reference checkout the reference library was built from, if any."""
    return os.path.realpath(REF_SOURCE_LINK) if os.path.isdir(REF_SOURCE_LINK) else None


def available(kind: str = "port") -> bool:
    return os.path.exists(PORT_SO if kind == "port" else REF_SO)


def _lib(kind: str) -> ctypes.CDLL:
    if kind in _libs:
        return _libs[kind]
    path = PORT_SO if kind == "port" else REF_SO
    if not os.path.exists(path):
        if kind == "port":
            build()
        else:
            raise FileNotFoundError(f"{path} not built (reference sources needed)")
    lib = ctypes.CDLL(path)
    pre = "oracle_" if kind == "port" else "ref_"
    f = getattr(lib, pre + "solve3d")
    f.restype = ctypes.c_int
    f.argtypes = [_ip, _ip, _dp, ctypes.c_int] + [ctypes.c_int] * 4 + [_dp] * 9
    if kind == "port":
        f = lib.oracle_solve3d_timed
        f.restype = ctypes.c_int
        f.argtypes = [_ip, _ip, _dp, ctypes.c_int] + [ctypes.c_int] * 4 + [_dp] * 10
    if kind == "port":
        f = lib.oracle_smooth3d
        f.restype = ctypes.c_int
        f.argtypes = [_ip, _ip, _dp, ctypes.c_double] + [_dp] * 6
        f = lib.oracle_gauss_green
        f.restype = ctypes.c_double
        f.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double]
        f = lib.oracle_solve3d_gauss
        f.restype = ctypes.c_int
        f.argtypes = [_ip, _ip, _dp, ctypes.c_int, ctypes.c_double] + [ctypes.c_int] * 4 + [_dp] * 9
        f = lib.oracle_solve2d_gauss
        f.restype = ctypes.c_int
        f.argtypes = [_ip, _ip, _dp, ctypes.c_int, ctypes.c_double] + [ctypes.c_int] * 3 + [_dp] * 9
    f = getattr(lib, pre + "solve2d")
    f.restype = ctypes.c_int
    f.argtypes = [_ip, _ip, _dp, ctypes.c_int] + [ctypes.c_int] * 3 + [_dp] * 9
    f = getattr(lib, pre + "greens3d")
    f.restype = ctypes.c_int
    f.argtypes = [_ip, _ip, _dp, ctypes.c_int, _dp, _dp, _dp, _ip]
    f = getattr(lib, pre + "fft")
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_int, ctypes.c_int, _dp]
    for name in ("sine_int", "bessel_int_J0"):
        f = getattr(lib, pre + name)
        f.restype = ctypes.c_double
        f.argtypes = [ctypes.c_double]
    _libs[kind] = lib
    return lib


def set_threads(n: int) -> int:
    """Threads of the port's solves (n <= 0: all cores); returns the count in use."""
    lib = _lib("port")
    lib.oracle_set_threads(ctypes.c_int(int(n)))
    lib.oracle_threads.restype = ctypes.c_int
    return int(lib.oracle_threads())


def _fn(kind: str, name: str):
    return getattr(_lib(kind), ("oracle_" if kind == "port" else "ref_") + name)


def _ptr(a):
    if a is None:
        return None
    return a.ctypes.data_as(_dp)


def _f64(a):
    if a is None:
        return None
    return np.ascontiguousarray(a, dtype=np.float64)


def sine_int(x: float, kind: str = "port") -> float:
    return _fn(kind, "sine_int")(float(x))


def bessel_int_J0(x: float, kind: str = "port") -> float:
    return _fn(kind, "bessel_int_J0")(float(x))


def fft(z: np.ndarray, inverse: bool = False, kind: str = "port") -> np.ndarray:
    """Unnormalised transform of a complex vector (forward e^{-2 pi i jk/n})."""
    z = np.ascontiguousarray(z, dtype=np.complex128).copy()
    buf = z.view(np.float64)
    st = _fn(kind, "fft")(z.size, 1 if inverse else -1, _ptr(buf))
    if st:
        raise RuntimeError(f"oracle fft status {st}")
    return z


def greens3d(ncell, bc, dx, reg: int = 0, kind: str = "port"):
    """(G complex [Pz][Py][Px], zeta [Pz][Py][Px] or None) as the kernel build makes them."""
    nc = (ctypes.c_int * 3)(*ncell)
    b = (ctypes.c_int * 3)(*bc)
    d = (ctypes.c_double * 3)(*dx)
    p = [(2 if bc[i] == 0 else 1) * ncell[i] for i in range(3)]
    n = p[0] * p[1] * p[2]
    gre = np.zeros(n)
    gim = np.zeros(n)
    zeta = np.zeros(n) if reg > 0 else None
    pext = (ctypes.c_int * 3)()
    st = _fn(kind, "greens3d")(nc, b, d, int(reg), _ptr(gre), _ptr(gim), _ptr(zeta), pext)
    if st:
        raise ValueError(f"oracle greens3d status {st}")
    shape = (p[2], p[1], p[0])
    g = (gre + 1j * gim).reshape(shape)
    return g, (zeta.reshape(shape) if zeta is not None else None)


def gauss_green(dim: int, m: int, s: float, r: float) -> float:
    """The Gaussian family's free-space kernel (dimension dim, order 2m, width s) at r."""
    return _lib("port").oracle_gauss_green(int(dim), int(m), float(s), float(r))


def solve3d(ncell, bc, dx, B, reg: int = 0, grad=False, div=False, curl=False,
            reproject=False, want_rhs=False, kind: str = "port", gauss_width: float | None = None):
    """Run setup3d/push/solve3d/pull. B: sequence of 3 arrays [Nz][Ny][Nx] or None.

    gauss_width (port only): solve with the Gaussian-regularised kernel family
    of that width (0: twice the largest cell size).
    Returns (A, RB): lists of 3 arrays or None (component not produced).
    """
    nx, ny, nz = ncell
    shape = (nz, ny, nx)
    Bc = [_f64(b) for b in B]
    for b in Bc:
        if b is not None and b.shape != shape:
            raise ValueError(f"field shape {b.shape} != {shape}")
    nan = float("nan")
    A = [np.full(shape, nan) for _ in range(3)]
    RB = [np.full(shape, nan) for _ in range(3)] if want_rhs else [None] * 3
    nc = (ctypes.c_int * 3)(*ncell)
    b = (ctypes.c_int * 3)(*bc)
    d = (ctypes.c_double * 3)(*dx)
    if gauss_width is None:
        st = _fn(kind, "solve3d")(nc, b, d, int(reg), int(grad), int(div), int(curl), int(reproject),
                                  *[_ptr(x) for x in Bc], *[_ptr(x) for x in A], *[_ptr(x) for x in RB])
    else:
        st = _lib("port").oracle_solve3d_gauss(nc, b, d, int(reg), float(gauss_width), int(grad), int(div),
                                               int(curl), int(reproject), *[_ptr(x) for x in Bc],
                                               *[_ptr(x) for x in A], *[_ptr(x) for x in RB])
    if st:
        raise ValueError(f"oracle solve3d status {st}")
    # components the solve did not produce stay NaN-filled: report them as None
    A = [a if not np.isnan(a).all() else None for a in A]
    RB = [r if (r is not None and not np.isnan(r).all()) else None for r in RB]
    return A, RB


def solve2d(ncell, bc, dx, B, reg: int = 0, grad=False, div=False, curl=False, want_rhs=False,
            kind: str = "port", gauss_width: float | None = None):
    """Run setup2d/push/solve2d/pull. B: sequence of 3 arrays [Ny][Nx] or None
    (X, Y and the out-of-plane Z). Returns (A, RB) as solve3d."""
    nx, ny = ncell
    shape = (ny, nx)
    Bc = [_f64(b) for b in B]
    for b in Bc:
        if b is not None and b.shape != shape:
            raise ValueError(f"field shape {b.shape} != {shape}")
    nan = float("nan")
    A = [np.full(shape, nan) for _ in range(3)]
    RB = [np.full(shape, nan) for _ in range(3)] if want_rhs else [None] * 3
    nc = (ctypes.c_int * 2)(*ncell)
    b = (ctypes.c_int * 2)(*bc)
    d = (ctypes.c_double * 2)(*dx)
    if gauss_width is None:
        st = _fn(kind, "solve2d")(nc, b, d, int(reg), int(grad), int(div), int(curl),
                                  *[_ptr(x) for x in Bc], *[_ptr(x) for x in A], *[_ptr(x) for x in RB])
    else:
        st = _lib("port").oracle_solve2d_gauss(nc, b, d, int(reg), float(gauss_width), int(grad), int(div),
                                               int(curl), *[_ptr(x) for x in Bc], *[_ptr(x) for x in A],
                                               *[_ptr(x) for x in RB])
    if st:
        raise ValueError(f"oracle solve2d status {st}")
    A = [a if not np.isnan(a).all() else None for a in A]
    RB = [r if (r is not None and not np.isnan(r).all()) else None for r in RB]
    return A, RB


def smooth3d(ncell, bc, dx, B, width: float):
    """Port of smooth3d: the fields B (3 arrays [Nz][Ny][Nx] or None), smoothed."""
    shape = (ncell[2], ncell[1], ncell[0])
    Bc = [_f64(b) for b in B]
    out = [None if b is None else np.empty(shape) for b in Bc]
    nc = (ctypes.c_int * 3)(*ncell)
    b = (ctypes.c_int * 3)(*bc)
    d = (ctypes.c_double * 3)(*dx)
    st = _lib("port").oracle_smooth3d(nc, b, d, float(width), *[_ptr(x) for x in Bc], *[_ptr(x) for x in out])
    if st:
        raise ValueError(f"oracle smooth3d status {st}")
    return out


def solve3d_timed(ncell, bc, dx, B, reg: int = 0, grad=False, div=False, curl=False, reproject=False):
    """Port solve returning (A, seconds[setup, push+solve, pull])."""
    nx, ny, nz = ncell
    shape = (nz, ny, nx)
    Bc = [_f64(b) for b in B]
    A = [np.empty(shape) for _ in range(3)]
    sec = np.zeros(3)
    nc = (ctypes.c_int * 3)(*ncell)
    b = (ctypes.c_int * 3)(*bc)
    d = (ctypes.c_double * 3)(*dx)
    st = _lib("port").oracle_solve3d_timed(nc, b, d, int(reg), int(grad), int(div), int(curl), int(reproject),
                                           *[_ptr(x) for x in Bc], *[_ptr(x) for x in A], None, None, None,
                                           _ptr(sec))
    if st:
        raise ValueError(f"oracle solve3d status {st}")
    return A, sec
