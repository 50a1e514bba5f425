"""Python mirror of the reference solver class (c++/source/poisson_solver.hpp:39-124).

Same member names and argument meaning as the reference C++ class --
setup3d/setup2d, set_return_grad/div/curl, set_reprojection, push,
solve3d/solve2d, pull and the ``partition`` list -- over the C ABI of
libps_gb300.so. Where the reference prints an error and returns, this raises
PSError with the same message. Fields are float64 arrays shaped (Nz, Ny, Nx)
(2D: (Ny, Nx)), x fastest, the layout the reference's push/pull use.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np

from . import _lib as L


@dataclass
class Partition:
    """One entry of the reference's ``partition`` vector (class_partition.hpp:29-43)."""
    ncell: tuple
    icell: tuple
    dx: tuple


def _check(lib, h, st):
    if st != L.PS_OK:
        msg = lib.ps_last_error(h)
        raise L.PSError(st, msg.decode() if msg else lib.ps_status_string(st).decode())


def _host_ptr(a, shape, name, writable=False):
    if a is None:
        return None
    if not isinstance(a, np.ndarray) or a.dtype != np.float64 or not a.flags.c_contiguous:
        raise TypeError(f"{name} must be a C-contiguous float64 numpy array")
    if a.shape != shape and a.size != int(np.prod(shape)):
        raise ValueError(f"{name} has shape {a.shape}, expected {shape}")
    if writable and not a.flags.writeable:
        raise ValueError(f"{name} is read-only")
    return a.ctypes.data


class PoissonSolver:
    """GB300 Green's-function FFT Poisson solver: lap(A) = -B in 3D or 2D."""

    def __init__(self):
        self._lib = L.load()
        h = ctypes.c_void_p()
        st = self._lib.ps_create(ctypes.byref(h))
        if st != L.PS_OK:
            raise L.PSError(st, self._lib.ps_status_string(st).decode())
        self._h = h
        self.partition: list[Partition] = []
        self._shape = None

    # -- lifetime --------------------------------------------------------
    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            self._lib.ps_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _call(self, name, *args):
        _check(self._lib, self._h, getattr(self._lib, name)(self._h, *args))

    # -- setup (setup3d.cpp:8-71) ---------------------------------------
    def setup3d(self, ncell, bc, dx, reg_order: int = 0):
        nc = (ctypes.c_int * 3)(*[int(v) for v in ncell])
        b = (ctypes.c_int * 3)(*[int(v) for v in bc])
        d = (ctypes.c_double * 3)(*[float(v) for v in dx])
        self._call("ps_setup3d", nc, b, d, int(reg_order))
        self._shape = (int(ncell[2]), int(ncell[1]), int(ncell[0]))
        self._fill_partition()

    def _fill_partition(self):
        self.partition = []
        for i in range(self._lib.ps_partition_count(self._h)):
            n3 = (ctypes.c_int * 3)()
            i3 = (ctypes.c_int * 3)()
            d3 = (ctypes.c_double * 3)()
            self._call("ps_partition", i, n3, i3, d3)
            self.partition.append(Partition(tuple(n3), tuple(i3), tuple(d3)))

    def setup2d(self, ncell, bc, dx, reg_order: int = 0):
        """2D solver (setup2d.cpp:8): fields are [Ny][Nx] arrays."""
        nc = (ctypes.c_int * 2)(*[int(v) for v in ncell])
        b = (ctypes.c_int * 2)(*[int(v) for v in bc])
        d = (ctypes.c_double * 2)(*[float(v) for v in dx])
        self._call("ps_setup2d", nc, b, d, int(reg_order))
        self._shape = (int(ncell[1]), int(ncell[0]))
        self._fill_partition()

    def solve2d(self):
        self._call("ps_solve2d")

    # -- options (settings.cpp:9-30) ------------------------------------
    def set_return_grad(self, toggle: bool):
        self._call("ps_set_option", L.PS_OPT_GRAD, int(bool(toggle)))

    def set_return_div(self, toggle: bool):
        self._call("ps_set_option", L.PS_OPT_DIV, int(bool(toggle)))

    def set_return_curl(self, toggle: bool):
        self._call("ps_set_option", L.PS_OPT_CURL, int(bool(toggle)))

    def set_reprojection(self, toggle: bool):
        self._call("ps_set_option", L.PS_OPT_REPROJECT, int(bool(toggle)))

    def set_precision(self, precision: str):
        """'fp64' (default), 'fp32' or 'df64' (double-float: pairs of FP32
        numbers, FP64-class accuracy) transforms; the kernel is always built
        in FP64."""
        v = {"fp64": L.PS_PREC_FP64, "fp32": L.PS_PREC_FP32, "df64": L.PS_PREC_DF64}[precision]
        self._call("ps_set_option", L.PS_OPT_PRECISION, v)

    def set_stream(self, stream_handle: int):
        self._call("ps_set_stream", ctypes.c_void_p(int(stream_handle)))

    def set_kernel(self, family: str, width: float = 0.0):
        """'spectral' (the reference's kernels, default) or 'gaussian': the
        Gaussian-regularised kernels of order max(2, reg_order) and width
        `width` (0: twice the largest cell size). On a set-up handle the
        kernel is rebuilt as a new setup."""
        v = {"spectral": L.PS_KERNEL_SPECTRAL, "gaussian": L.PS_KERNEL_GAUSSIAN}[family]
        self._call("ps_set_kernel", v, float(width))

    # -- host push / solve / pull ----------------------------------------
    def push(self, bx, by=None, bz=None):
        s = self._shape
        self._call("ps_push", _host_ptr(bx, s, "Bx"), _host_ptr(by, s, "By"), _host_ptr(bz, s, "Bz"))

    def solve3d(self):
        self._call("ps_solve3d")

    def pull(self, ax=None, ay=None, az=None, bx=None, by=None, bz=None):
        s = self._shape
        ptrs = [_host_ptr(a, s, n, True) for a, n in zip((ax, ay, az, bx, by, bz),
                                                         ("Ax", "Ay", "Az", "Bx", "By", "Bz"))]
        self._call("ps_pull", *ptrs)

    # -- Fortran-style interleaved arrays (poisson_solver_push.f / pull.f) ----
    def push_interleaved(self, b, offset=(0, 0, 0)):
        """b: float64 array shaped (ext_z, ext_y, ext_x, ncomp), ncomp 1..3
        (X; X, Y; X, Y, Z); the field box starts at offset (x, y, z)."""
        b = np.ascontiguousarray(b, dtype=np.float64)
        ext = (ctypes.c_int * 3)(b.shape[2], b.shape[1], b.shape[0])
        off = (ctypes.c_int * 3)(*[int(v) for v in offset])
        self._call("ps_push_interleaved", b.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), int(b.shape[3]), ext, off)

    def pull_interleaved(self, a=None, b=None, offset=(0, 0, 0)):
        """Write the solution into a and the returned right-hand side into b,
        arrays shaped (ext_z, ext_y, ext_x, ncomp) (either may be None)."""
        ref = a if a is not None else b
        if ref is None:
            return
        for arr in (a, b):
            if arr is not None and (arr.dtype != np.float64 or not arr.flags.c_contiguous or arr.ndim != 4
                                    or arr.shape[:3] != ref.shape[:3]):
                raise TypeError("interleaved arrays must be C-contiguous float64 (ext_z, ext_y, ext_x, ncomp) alike")
        ext = (ctypes.c_int * 3)(ref.shape[2], ref.shape[1], ref.shape[0])
        off = (ctypes.c_int * 3)(*[int(v) for v in offset])
        dp = ctypes.POINTER(ctypes.c_double)
        self._call("ps_pull_interleaved", None if a is None else a.ctypes.data_as(dp), 0 if a is None else a.shape[3],
                   None if b is None else b.ctypes.data_as(dp), 0 if b is None else b.shape[3], ext, off)

    def smooth3d(self, width: float):
        """Gaussian smoothing of the pushed fields, exp(-width^2 |k|^2 / 2), in place."""
        self._call("ps_smooth3d", float(width))

    # -- device pointers (raw CUDA addresses, e.g. torch tensor.data_ptr()) --
    def push_device(self, bx, by=0, bz=0):
        self._call("ps_push_device", bx or None, by or None, bz or None)

    def pull_device(self, ax=0, ay=0, az=0, bx=0, by=0, bz=0):
        self._call("ps_pull_device", *[p or None for p in (ax, ay, az, bx, by, bz)])

    def solve3d_device(self, b_ptrs, a_ptrs):
        """One device-resident solve: b_ptrs / a_ptrs are 3 addresses (0 = absent)."""
        self._call("ps_solve3d_device", *[p or None for p in b_ptrs], *[p or None for p in a_ptrs])

    def set_pass_timing(self, on: bool):
        self._call("ps_set_option", L.PS_OPT_PASS_TIMING, int(bool(on)))

    def pass_times(self, reset: bool = True):
        """(per-pass milliseconds summed over timed solves, number of solves)."""
        ms = (ctypes.c_double * 5)()
        n = ctypes.c_int()
        self._call("ps_get_pass_times", ms, ctypes.byref(n), int(reset))
        return list(ms), n.value

    def autotune(self, component_mask: int = 7):
        """Time each pass's kernel families and lines per CTA; keep the fastest."""
        self._call("ps_autotune", int(component_mask))

    def pass_config(self, component_mask: int = 7):
        """[(family name, lines per CTA)] of the five passes a solve would run."""
        out = []
        for p in range(5):
            f, b = ctypes.c_int(), ctypes.c_int()
            self._call("ps_get_pass_config", p, int(component_mask), ctypes.byref(f), ctypes.byref(b))
            out.append((L.FAMILY_NAMES[f.value], b.value))
        return out

    def pass_plan(self, component_mask: int = 7):
        """[(stage radices, Bluestein convolution length or 0)] of the five
        passes a solve would run."""
        out = []
        for p in range(5):
            rad = (ctypes.c_int * 16)()
            ns, m = ctypes.c_int(), ctypes.c_int()
            self._call("ps_get_pass_plan", p, int(component_mask), rad, 16, ctypes.byref(ns), ctypes.byref(m))
            out.append((list(rad[:min(ns.value, 16)]), m.value))
        return out

    def synchronize(self):
        self._call("ps_synchronize")

    # -- introspection -----------------------------------------------------
    def info(self, what: int) -> float:
        v = ctypes.c_double()
        _check(self._lib, self._h, self._lib.ps_get_info(self._h, what, ctypes.byref(v)))
        return v.value

    def kernel_octant(self) -> np.ndarray:
        """FP64 octant K = G zeta / (Px Py Pz), shape (Pz/2+1, Py/2+1, Px/2+1)."""
        p = [int(self.info(w)) for w in (L.PS_INFO_PADDED_X, L.PS_INFO_PADDED_Y, L.PS_INFO_PADDED_Z)]
        out = np.empty((p[2] // 2 + 1, p[1] // 2 + 1, p[0] // 2 + 1))
        self._call("ps_get_kernel", out.ctypes.data, out.size)
        return out

    @property
    def padded(self):
        return tuple(int(self.info(w)) for w in (L.PS_INFO_PADDED_X, L.PS_INFO_PADDED_Y, L.PS_INFO_PADDED_Z))


class PoissonBatch:
    """Many independent problems solved together (no single reference call:
    the reference holds one poisson_solver object per problem).

    ``add`` stands for setup3d of one problem and returns its index;
    ``push``/``pull``/``set_return_*`` take that index first. ``solve`` runs
    every problem with one launch per pass, replayed through a CUDA graph.
    """

    def __init__(self, precision: str = "fp64"):
        self._lib = L.load()
        prec = {"fp64": L.PS_PREC_FP64, "fp32": L.PS_PREC_FP32, "df64": L.PS_PREC_DF64}[precision]
        h = ctypes.c_void_p()
        st = self._lib.ps_batch_create(ctypes.byref(h), prec)
        if st != L.PS_OK:
            raise L.PSError(st, self._lib.ps_status_string(st).decode())
        self._h = h
        self._shapes: list[tuple] = []

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            self._lib.ps_batch_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __len__(self):
        return len(self._shapes)

    def _call(self, name, *args):
        st = getattr(self._lib, name)(self._h, *args)
        if st != L.PS_OK:
            msg = self._lib.ps_batch_last_error(self._h)
            raise L.PSError(st, msg.decode() if msg else self._lib.ps_status_string(st).decode())

    def add(self, ncell, bc, dx, reg_order: int = 0) -> int:
        nc = (ctypes.c_int * 3)(*[int(v) for v in ncell])
        b = (ctypes.c_int * 3)(*[int(v) for v in bc])
        d = (ctypes.c_double * 3)(*[float(v) for v in dx])
        idx = ctypes.c_int()
        self._call("ps_batch_add", nc, b, d, int(reg_order), ctypes.byref(idx))
        self._shapes.append((int(ncell[2]), int(ncell[1]), int(ncell[0])))
        return idx.value

    def set_return_grad(self, i: int, toggle: bool):
        self._call("ps_batch_set_option", int(i), L.PS_OPT_GRAD, int(bool(toggle)))

    def set_return_div(self, i: int, toggle: bool):
        self._call("ps_batch_set_option", int(i), L.PS_OPT_DIV, int(bool(toggle)))

    def set_return_curl(self, i: int, toggle: bool):
        self._call("ps_batch_set_option", int(i), L.PS_OPT_CURL, int(bool(toggle)))

    def set_kernel(self, i: int, family: str, width: float = 0.0):
        """Kernel family of problem i ('spectral' or 'gaussian'); push after it."""
        v = {"spectral": L.PS_KERNEL_SPECTRAL, "gaussian": L.PS_KERNEL_GAUSSIAN}[family]
        self._call("ps_batch_set_kernel", int(i), v, float(width))

    def set_reprojection(self, i: int, toggle: bool):
        self._call("ps_batch_set_option", int(i), L.PS_OPT_REPROJECT, int(bool(toggle)))

    def push(self, i: int, bx, by=None, bz=None):
        s = self._shapes[i]
        self._call("ps_batch_push", int(i), _host_ptr(bx, s, "Bx"), _host_ptr(by, s, "By"), _host_ptr(bz, s, "Bz"))

    def push_device(self, i: int, bx, by=0, bz=0):
        self._call("ps_batch_push_device", int(i), bx or None, by or None, bz or None)

    def solve(self):
        self._call("ps_batch_solve")

    def autotune(self):
        """Time the plan variants (FP32) and the batched launches' shapes on
        the pushed problems and keep the fastest."""
        self._call("ps_batch_autotune")

    def set_tuning(self, axis: int, max_threads: int, start_lines: int, plan_variant: int):
        """Set the CTA thread bound, starting lines and plan variant of the x
        (0), y (1) or z (2) launches; the next solve rebuilds the batch."""
        self._call("ps_batch_set_tuning", int(axis), int(max_threads), int(start_lines), int(plan_variant))

    def tuning(self):
        """[(CTA thread bound, starting lines, plan variant)] of the x, y and
        z launches."""
        out = []
        for ax in range(3):
            t, s, v = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
            self._call("ps_batch_get_tuning", ax, ctypes.byref(t), ctypes.byref(s), ctypes.byref(v))
            out.append((t.value, s.value, v.value))
        return out

    def pull(self, i: int, ax=None, ay=None, az=None):
        s = self._shapes[i]
        self._call("ps_batch_pull", int(i), _host_ptr(ax, s, "Ax", True), _host_ptr(ay, s, "Ay", True),
                   _host_ptr(az, s, "Az", True))

    def pull_device(self, i: int, ax=0, ay=0, az=0):
        self._call("ps_batch_pull_device", int(i), ax or None, ay or None, az or None)

    def set_stream(self, stream_handle: int):
        self._call("ps_batch_set_stream", ctypes.c_void_p(int(stream_handle)))

    def synchronize(self):
        self._call("ps_batch_synchronize")

    def info(self, what: int) -> float:
        v = ctypes.c_double()
        st = self._lib.ps_batch_get_info(self._h, int(what), ctypes.byref(v))
        if st != L.PS_OK:
            raise L.PSError(st, self._lib.ps_status_string(st).decode())
        return v.value


def solve2d(ncell, bc, dx, B, reg_order=0, grad=False, div=False, curl=False,
            precision="fp64", want_rhs=False, kernel="spectral", width=0.0):
    """One-shot host 2D solve; B: 3 arrays [Ny][Nx] or None (X, Y, Z).
    Returns (A, RB) lists of 3 arrays or None."""
    shape = (ncell[1], ncell[0])
    with PoissonSolver() as ps:
        ps.set_kernel(kernel, width)
        ps.setup2d(ncell, bc, dx, reg_order)
        ps.set_return_grad(grad)
        ps.set_return_div(div)
        ps.set_return_curl(curl)
        ps.set_precision(precision)
        Bc = [None if b is None else np.ascontiguousarray(b, dtype=np.float64) for b in B]
        ps.push(*Bc)
        ps.solve2d()
        nan = float("nan")
        A = [np.full(shape, nan) for _ in range(3)]
        RB = [np.full(shape, nan) for _ in range(3)] if want_rhs else [None] * 3
        ps.pull(*A, *RB)
    A = [a if not np.isnan(a).all() else None for a in A]
    RB = [r if (r is not None and not np.isnan(r).all()) else None for r in RB]
    return A, RB


def solve(ncell, bc, dx, B, reg_order=0, grad=False, div=False, curl=False,
          reproject=False, precision="fp64", want_rhs=False, kernel="spectral", width=0.0):
    """One-shot host solve; returns (A, RB) lists of 3 arrays or None."""
    shape = (ncell[2], ncell[1], ncell[0])
    with PoissonSolver() as ps:
        ps.set_kernel(kernel, width)
        ps.setup3d(ncell, bc, dx, reg_order)
        ps.set_return_grad(grad)
        ps.set_return_div(div)
        ps.set_return_curl(curl)
        ps.set_reprojection(reproject)
        ps.set_precision(precision)
        Bc = [None if b is None else np.ascontiguousarray(b, dtype=np.float64) for b in B]
        ps.push(*Bc)
        ps.solve3d()
        nan = float("nan")
        A = [np.full(shape, nan) for _ in range(3)]
        RB = [np.full(shape, nan) for _ in range(3)] if want_rhs else [None] * 3
        ps.pull(*A, *RB)
    A = [a if not np.isnan(a).all() else None for a in A]
    RB = [r if (r is not None and not np.isnan(r).all()) else None for r in RB]
    return A, RB
