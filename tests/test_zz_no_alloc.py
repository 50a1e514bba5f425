"""ps_solve3d_device_noalloc: the solve for callers that may not allocate
device memory while they run (for example a time-stepping code whose device
memory budget is fixed before the loop starts). It must give the results of
ps_solve3d_device, call after call, while leaving the device's free memory
unchanged, and refuse problems larger than its fixed 32 MiB of scratch.

This file is collected last on purpose, so a run that stops at the first
failure has already run every other test.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12


def _setup(lib, ncell, bc, dx, reg, option):
    h = ctypes.c_void_p()
    assert lib.ps_create(ctypes.byref(h)) == 0
    st = lib.ps_setup3d(h, (ctypes.c_int * 3)(*ncell), (ctypes.c_int * 3)(*bc), (ctypes.c_double * 3)(*dx), reg)
    assert st == 0, lib.ps_last_error(h)
    if option is not None:
        assert lib.ps_set_option(h, option, 1) == 0
    return h


def _rel(a, b):
    import torch
    num = sum(float(torch.sum((x - y) ** 2)) for x, y in zip(a, b))
    den = sum(float(torch.sum(y ** 2)) for y in b)
    return (num / den) ** 0.5


@pytest.mark.parametrize("case", [
    ((24, 20, 16), (0, 0, 0), (0.1, 0.12, 0.15), 2, "curl", 3),
    ((18, 14, 22), (1, 1, 0), (0.1, 0.1, 0.1), 0, "grad", 1),
    ((16, 12, 10), (0, 0, 1), (0.2, 0.1, 0.1), 4, None, 2),
])
def test_noalloc_matches_device_solve_on_two_calls(native, case):
    torch = pytest.importorskip("torch")
    from poisson_solver_gb300 import _lib
    lib = _lib.load()
    ncell, bc, dx, reg, opt, ncomp = case
    option = {"curl": _lib.PS_OPT_CURL, "grad": _lib.PS_OPT_GRAD, None: None}[opt]
    h = _setup(lib, ncell, bc, dx, reg, option)
    dev = torch.device("cuda:0")
    shape = (ncell[2], ncell[1], ncell[0])
    gen = torch.Generator(device="cpu").manual_seed(sum(ncell))
    B = [torch.randn(shape, generator=gen, dtype=torch.float64).to(dev) if c < ncomp else None for c in range(3)]
    if bc == (1, 1, 0):
        B = [b - b.mean(dim=(1, 2), keepdim=True) if b is not None else None for b in B]
    bp = [b.data_ptr() if b is not None else None for b in B]
    nout = 3 if opt in ("curl", "grad") else ncomp
    ref = [torch.empty(shape, dtype=torch.float64, device=dev) for _ in range(nout)]
    ap = [a.data_ptr() for a in ref] + [None] * (3 - nout)
    assert lib.ps_solve3d_device(h, *bp, *ap) == 0, lib.ps_last_error(h)
    torch.cuda.synchronize()

    for call in range(2):
        out = [torch.full(shape, float("nan"), dtype=torch.float64, device=dev) for _ in range(nout)]
        op = [a.data_ptr() for a in out] + [None] * (3 - nout)
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info(0)[0]
        st = lib.ps_solve3d_device_noalloc(h, *bp, *op)
        assert st == 0, lib.ps_last_error(h)
        torch.cuda.synchronize()
        free_after = torch.cuda.mem_get_info(0)[0]
        assert _rel(out, ref) < FP64_TOL, f"call {call}"
        if call == 1:  # the first call may load this part of the library's device code
            assert free_after == free_before
    lib.ps_destroy(h)


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
