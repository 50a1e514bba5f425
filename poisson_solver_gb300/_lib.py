"""ctypes binding of the C ABI declared in include/poisson_solver_gb300.h.

The library is built in-tree (poisson_solver_gb300/libps_gb300.so, see
build.py). There is no fallback: if the library is missing or fails to load,
every call raises.
"""
from __future__ import annotations

import ctypes
import os

from .build import LIB

PS_OK = 0
PS_ERR_ARGUMENT = 1
PS_ERR_BOUNDARY = 2
PS_ERR_COMPONENTS = 3
PS_ERR_MEMORY = 4
PS_ERR_CUDA = 5
PS_ERR_STATE = 6
PS_ERR_UNSUPPORTED = 7
PS_ERR_TIMEOUT = 8

PS_OPT_GRAD = 0
PS_OPT_DIV = 1
PS_OPT_CURL = 2
PS_OPT_REPROJECT = 3
PS_OPT_PRECISION = 4
PS_OPT_PASS_TIMING = 5

PS_PREC_FP64 = 0
PS_PREC_FP32 = 1
PS_PREC_DF64 = 2

PS_KERNEL_SPECTRAL = 0
PS_KERNEL_GAUSSIAN = 1

PS_INFO_PADDED_X = 0
PS_INFO_PADDED_Y = 1
PS_INFO_PADDED_Z = 2
PS_INFO_LAUNCHES_PER_SOLVE = 3
PS_INFO_DEVICE_BYTES = 4
PS_INFO_KERNEL_OCTANT = 5

PS_FAMILY_RUNTIME = 0
PS_FAMILY_P2 = 1
PS_FAMILY_WIDE = 2
PS_FAMILY_TMEM = 3
PS_FAMILY_TMA = 4
FAMILY_NAMES = {0: "runtime", 1: "p2", 2: "wide", 3: "tmem", 4: "tma", 5: "tc"}

PS_BATCH_INFO_LAUNCHES_PER_SOLVE = 0
PS_BATCH_INFO_TILES_PER_SOLVE = 1
PS_BATCH_INFO_POINTS = 2
PS_BATCH_INFO_KERNEL_BUILDS = 3

# Every symbol the header declares, with (restype, argtypes).
_vp = ctypes.c_void_p
_ip = ctypes.POINTER(ctypes.c_int)
_dp = ctypes.c_void_p  # double* passed as raw addresses (host or device)
_i = ctypes.c_int
SIGNATURES = {
    "ps_create": (_i, [ctypes.POINTER(_vp)]),
    "ps_destroy": (_i, [_vp]),
    "ps_setup3d": (_i, [_vp, _ip, _ip, ctypes.POINTER(ctypes.c_double), _i]),
    "ps_set_option": (_i, [_vp, _i, _i]),
    "ps_get_option": (_i, [_vp, _i, _ip]),
    "ps_push": (_i, [_vp, _dp, _dp, _dp]),
    "ps_push_interleaved": (_i, [_vp, _dp, _i, _ip, _ip]),
    "ps_pull_interleaved": (_i, [_vp, _dp, _i, _dp, _i, _ip, _ip]),
    "ps_smooth3d": (_i, [_vp, ctypes.c_double]),
    "ps_set_kernel": (_i, [_vp, _i, ctypes.c_double]),
    "ps_solve3d": (_i, [_vp]),
    "ps_pull": (_i, [_vp, _dp, _dp, _dp, _dp, _dp, _dp]),
    "ps_push_device": (_i, [_vp, _dp, _dp, _dp]),
    "ps_pull_device": (_i, [_vp, _dp, _dp, _dp, _dp, _dp, _dp]),
    "ps_solve3d_device": (_i, [_vp, _dp, _dp, _dp, _dp, _dp, _dp]),
    "ps_solve3d_device_noalloc": (_i, [_vp, _dp, _dp, _dp, _dp, _dp, _dp]),
    "ps_partition_count": (_i, [_vp]),
    "ps_partition": (_i, [_vp, _i, _ip, _ip, ctypes.POINTER(ctypes.c_double)]),
    "ps_setup2d": (_i, [_vp, _ip, _ip, ctypes.POINTER(ctypes.c_double), _i]),
    "ps_solve2d": (_i, [_vp]),
    "ps_set_stream": (_i, [_vp, _vp]),
    "ps_synchronize": (_i, [_vp]),
    "ps_last_error": (ctypes.c_char_p, [_vp]),
    "ps_status_string": (ctypes.c_char_p, [_i]),
    "ps_get_info": (_i, [_vp, _i, ctypes.POINTER(ctypes.c_double)]),
    "ps_get_kernel": (_i, [_vp, _dp, ctypes.c_longlong]),
    "ps_get_pass_times": (_i, [_vp, ctypes.POINTER(ctypes.c_double), _ip, _i]),
    "ps_autotune": (_i, [_vp, _i]),
    "ps_get_pass_config": (_i, [_vp, _i, _i, _ip, _ip]),
    "ps_get_pass_plan": (_i, [_vp, _i, _i, _ip, _i, _ip, _ip]),
    "ps_batch_create": (_i, [ctypes.POINTER(_vp), _i]),
    "ps_batch_destroy": (_i, [_vp]),
    "ps_batch_add": (_i, [_vp, _ip, _ip, ctypes.POINTER(ctypes.c_double), _i, _ip]),
    "ps_batch_count": (_i, [_vp, _ip]),
    "ps_batch_set_option": (_i, [_vp, _i, _i, _i]),
    "ps_batch_set_kernel": (_i, [_vp, _i, _i, ctypes.c_double]),
    "ps_batch_push": (_i, [_vp, _i, _dp, _dp, _dp]),
    "ps_batch_push_device": (_i, [_vp, _i, _dp, _dp, _dp]),
    "ps_batch_solve": (_i, [_vp]),
    "ps_batch_autotune": (_i, [_vp]),
    "ps_batch_get_tuning": (_i, [_vp, _i, _ip, _ip, _ip]),
    "ps_batch_set_tuning": (_i, [_vp, _i, _i, _i, _i]),
    "ps_batch_pull": (_i, [_vp, _i, _dp, _dp, _dp]),
    "ps_batch_pull_device": (_i, [_vp, _i, _dp, _dp, _dp]),
    "ps_batch_set_stream": (_i, [_vp, _vp]),
    "ps_batch_synchronize": (_i, [_vp]),
    "ps_batch_get_info": (_i, [_vp, _i, ctypes.POINTER(ctypes.c_double)]),
    "ps_batch_last_error": (ctypes.c_char_p, [_vp]),
}

_lib: ctypes.CDLL | None = None


class PSError(RuntimeError):
    """A C-ABI call returned a non-zero status."""

    def __init__(self, status: int, message: str):
        super().__init__(f"[status {status}] {message}")
        self.status = status
        self.message = message


def lib_path() -> str:
    return os.environ.get("PS_GB300_LIB", LIB)


def load() -> ctypes.CDLL:
    """Load the native library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    path = lib_path()
    if not os.path.exists(path):
        raise ImportError(
            f"native library {path} is missing: build it with "
            "`python -c 'import __graft_entry__ as g; g.build()'` or `python -m poisson_solver_gb300.build`")
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib
