"""ps_solve3d_device_noalloc: the solve for callers that may not allocate
device memory while they run (for example a time-stepping code whose device
memory budget is fixed before the loop starts). It must give the oracle's
results and those of ps_solve3d_device, call after call, while leaving the
device's free memory unchanged, and refuse problems larger than its fixed
32 MiB of scratch.

This file is collected last on purpose, so a run that stops at the first
failure has already run every other test.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12


def _setup(lib, ncell, bc, dx, reg, option, precision=None):
    from poisson_solver_gb300 import _lib
    h = ctypes.c_void_p()
    assert lib.ps_create(ctypes.byref(h)) == 0
    st = lib.ps_setup3d(h, (ctypes.c_int * 3)(*ncell), (ctypes.c_int * 3)(*bc), (ctypes.c_double * 3)(*dx), reg)
    assert st == 0, lib.ps_last_error(h)
    if option is not None:
        assert lib.ps_set_option(h, option, 1) == 0
    if precision is not None:
        assert lib.ps_set_option(h, _lib.PS_OPT_PRECISION, precision) == 0
    return h


def _rel(a, b):
    num = sum(float(np.sum((np.asarray(x) - np.asarray(y)) ** 2)) for x, y in zip(a, b))
    den = sum(float(np.sum(np.asarray(y) ** 2)) for y in b)
    return (num / den) ** 0.5


def _inputs(ncell, bc, ncomp):
    shape = (ncell[2], ncell[1], ncell[0])
    rng = np.random.default_rng(sum(ncell))
    B = [rng.standard_normal(shape) if c < ncomp else None for c in range(3)]
    if bc == (1, 1, 0):  # zero x-y mean: the periodic-periodic-unbounded kernel's k = 0 line
        B = [b - b.mean(axis=(1, 2), keepdims=True) if b is not None else None for b in B]
    return B


CASES = [
    ((24, 20, 16), (0, 0, 0), (0.1, 0.12, 0.15), 2, "curl", 3),
    ((18, 14, 22), (1, 1, 0), (0.1, 0.1, 0.1), 0, "grad", 1),
    ((16, 12, 10), (0, 0, 1), (0.2, 0.1, 0.1), 4, None, 2),
    # padded x length 34 = 2 x 17: the Bluestein plan
    ((17, 12, 10), (0, 0, 0), (0.1, 0.1, 0.1), 2, "curl", 3),
]


@pytest.mark.parametrize("case", CASES)
def test_noalloc_matches_oracle_and_device_solve_on_two_calls(native, oracle, case):
    torch = pytest.importorskip("torch")
    from poisson_solver_gb300 import _lib
    lib = _lib.load()
    ncell, bc, dx, reg, opt, ncomp = case
    option = {"curl": _lib.PS_OPT_CURL, "grad": _lib.PS_OPT_GRAD, None: None}[opt]
    Bh = _inputs(ncell, bc, ncomp)
    want, _ = oracle.solve3d(ncell, bc, dx, Bh, reg=reg, curl=opt == "curl", grad=opt == "grad")
    want = [a for a in want if a is not None]

    h = _setup(lib, ncell, bc, dx, reg, option)
    dev = torch.device("cuda:0")
    shape = (ncell[2], ncell[1], ncell[0])
    B = [torch.from_numpy(b).to(dev) if b is not None else None for b in Bh]
    bp = [b.data_ptr() if b is not None else None for b in B]
    nout = len(want)
    ref = [torch.empty(shape, dtype=torch.float64, device=dev) for _ in range(nout)]
    ap = [a.data_ptr() for a in ref] + [None] * (3 - nout)
    assert lib.ps_solve3d_device(h, *bp, *ap) == 0, lib.ps_last_error(h)
    torch.cuda.synchronize()
    ref = [a.cpu().numpy() for a in ref]

    for call in range(2):
        out = [torch.full(shape, float("nan"), dtype=torch.float64, device=dev) for _ in range(nout)]
        op = [a.data_ptr() for a in out] + [None] * (3 - nout)
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info(0)[0]
        st = lib.ps_solve3d_device_noalloc(h, *bp, *op)
        assert st == 0, lib.ps_last_error(h)
        torch.cuda.synchronize()
        free_after = torch.cuda.mem_get_info(0)[0]
        got = [a.cpu().numpy() for a in out]
        assert _rel(got, want) < FP64_TOL, f"call {call} vs oracle"
        assert _rel(got, ref) < FP64_TOL, f"call {call} vs ps_solve3d_device"
        if call == 1:  # the first call may load this part of the library's device code
            assert free_after == free_before
    lib.ps_destroy(h)


def test_noalloc_transforms_in_fp64_on_an_fp32_handle(native):
    """The handle's precision option does not reach this entry point: on a
    handle set to FP32 transforms it still gives the FP64 solve."""
    torch = pytest.importorskip("torch")
    from poisson_solver_gb300 import _lib
    lib = _lib.load()
    ncell, bc, dx, reg = (20, 16, 12), (0, 0, 0), (0.1, 0.1, 0.1), 2
    Bh = _inputs(ncell, bc, 3)
    dev = torch.device("cuda:0")
    shape = (ncell[2], ncell[1], ncell[0])
    B = [torch.from_numpy(b).to(dev) for b in Bh]
    bp = [b.data_ptr() for b in B]
    h64 = _setup(lib, ncell, bc, dx, reg, _lib.PS_OPT_CURL)
    h32 = _setup(lib, ncell, bc, dx, reg, _lib.PS_OPT_CURL, precision=_lib.PS_PREC_FP32)
    ref = [torch.empty(shape, dtype=torch.float64, device=dev) for _ in range(3)]
    assert lib.ps_solve3d_device(h64, *bp, *[a.data_ptr() for a in ref]) == 0, lib.ps_last_error(h64)
    for _ in range(2):
        out = [torch.full(shape, float("nan"), dtype=torch.float64, device=dev) for _ in range(3)]
        assert lib.ps_solve3d_device_noalloc(h32, *bp, *[a.data_ptr() for a in out]) == 0, lib.ps_last_error(h32)
        torch.cuda.synchronize()
        assert _rel([a.cpu().numpy() for a in out], [a.cpu().numpy() for a in ref]) < FP64_TOL
    lib.ps_destroy(h64)
    lib.ps_destroy(h32)


def test_noalloc_rejects_problems_above_its_scratch(native):
    torch = pytest.importorskip("torch")
    from poisson_solver_gb300 import _lib
    lib = _lib.load()
    h = _setup(lib, (128, 128, 128), (0, 0, 0), (1 / 64,) * 3, 0, None)
    b = torch.zeros((128, 128, 128), dtype=torch.float64, device="cuda:0")
    a = torch.empty_like(b)
    st = lib.ps_solve3d_device_noalloc(h, b.data_ptr(), None, None, a.data_ptr(), None, None)
    assert st == _lib.PS_ERR_UNSUPPORTED
    msg = lib.ps_last_error(h).decode()
    assert "33554432 bytes of scratch" in msg and "needs" in msg
    lib.ps_destroy(h)
