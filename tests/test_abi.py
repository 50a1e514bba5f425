"""The C ABI library without a GPU: it loads, exports every symbol the header
declares, and the drop-in C++ header compiles and links against it."""
import ctypes
import os
import re
import shutil
import subprocess

import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "poisson_solver_gb300.h")


def ref_tests_dir():
    """The reference's own test programs, where the oracle build found the reference."""
    from oracle import oracle
    root = os.environ.get("PS_REFERENCE_ROOT") or oracle.reference_root()
    return os.path.join(root, "c++", "test") if root else None


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(ps_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_the_abi():
    names = declared_functions()
    for required in ("ps_create", "ps_destroy", "ps_setup3d", "ps_set_option", "ps_push", "ps_solve3d",
                     "ps_pull", "ps_partition", "ps_last_error", "ps_solve3d_device"):
        assert required in names


def test_library_exports_every_declared_symbol(native):
    from poisson_solver_gb300 import _lib
    lib = _lib.load()
    for name in declared_functions():
        assert hasattr(lib, name), name
        assert name in _lib.SIGNATURES, f"{name} has no ctypes signature"
    out = subprocess.run(["nm", "-D", "--defined-only", _lib.lib_path()], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\bT (ps_[a-z0-9_]+)", out))
    assert exported == set(declared_functions())


def test_status_strings_and_null_handles(native):
    from poisson_solver_gb300 import _lib
    lib = _lib.load()
    assert lib.ps_status_string(0) == b"ok"
    assert lib.ps_status_string(3).startswith(b"pushed components")
    assert b"timed out" in lib.ps_status_string(_lib.PS_ERR_TIMEOUT)
    assert lib.ps_solve3d(None) == _lib.PS_ERR_ARGUMENT
    assert lib.ps_destroy(None) == _lib.PS_OK
    assert lib.ps_setup2d(None, None, None, None, 0) == _lib.PS_ERR_ARGUMENT
    assert lib.ps_partition_count(None) == 0
    # the Fortran-style entry points and the kernel family check the handle first
    ext = (ctypes.c_int * 3)(4, 4, 4)
    off = (ctypes.c_int * 3)(0, 0, 0)
    assert lib.ps_push_interleaved(None, None, 1, ext, off) == _lib.PS_ERR_ARGUMENT
    assert lib.ps_pull_interleaved(None, None, 1, None, 0, ext, off) == _lib.PS_ERR_ARGUMENT
    assert lib.ps_smooth3d(None, 0.1) == _lib.PS_ERR_ARGUMENT
    assert lib.ps_set_kernel(None, _lib.PS_KERNEL_GAUSSIAN, 0.0) == _lib.PS_ERR_ARGUMENT


DROPIN_CLIENT = r"""
#include "mpi.h"
#include "poisson_solver.hpp"
// Client code in the shape of the reference's validation programs.
int main(int argc, char** argv) {
  MPI_Init(&argc, &argv);
  int rank = 0; MPI_Comm_rank(MPI_COMM_WORLD, &rank);
  int ncell[3] = {16, 16, 16}; int bc[3] = {0, 0, 0}; double dx[3] = {0.125, 0.125, 0.125};
  poisson_solver poisson;
  poisson.setup3d(ncell, bc, dx);
  poisson.set_return_curl(true);
  int n = poisson.partition[rank].ncell[0] * poisson.partition[rank].ncell[1] * poisson.partition[rank].ncell[2];
  double *B[3], *A[3];
  for (int c = 0; c < 3; ++c) { B[c] = new double[n](); A[c] = new double[n](); }
  poisson.push(B[0], B[1], B[2]);
  poisson.solve3d();
  poisson.pull(A[0], A[1], A[2], B[0], B[1], B[2]);
  // the extensions: double-float transforms, kernel family, interleaved
  // ghost-offset arrays, smoothing
  poisson.set_precision(PS_PREC_DF64);
  poisson.solve3d();
  poisson.pull(A[0], A[1], A[2], nullptr, nullptr, nullptr);
  int ext[3] = {20, 18, 16}, off[3] = {2, 1, 0};
  double *I = new double[3 * 20 * 18 * 16]();
  poisson.set_kernel(PS_KERNEL_GAUSSIAN);
  poisson.push_interleaved(I, 3, ext, off);
  poisson.smooth3d(0.2);
  poisson.solve3d();
  poisson.pull_interleaved(I, 3, nullptr, 0, ext, off);
  MPI_Finalize();
  return poisson.last_status();
}
"""


def test_dropin_header_compiles_and_links(native, tmp_path):
    from poisson_solver_gb300 import _lib
    src = tmp_path / "client.cpp"
    src.write_text(DROPIN_CLIENT)
    exe = tmp_path / "client"
    cmd = ["g++", "-std=c++11", "-O1", "-I", os.path.join(ROOT, "include"), "-I", os.path.join(ROOT, "oracle", "mpi_stub"),
           str(src), "-o", str(exe), _lib.lib_path(), f"-Wl,-rpath,{os.path.dirname(_lib.lib_path())}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


@pytest.mark.parametrize("prog", ["unbounded3d", "periodic3d", "mixed_ppf3d", "mixed_ffp3d",
                                  "unbounded2d", "periodic2d", "mixed2d"])
def test_reference_validation_programs_build_unchanged(native, oracle, tmp_path, prog):
    """The reference's own 3D and 2D test programs compile and link, unmodified, against the drop-in."""
    tests_dir = ref_tests_dir()
    src = os.path.join(tests_dir, prog, "sources", "main.cpp") if tests_dir else ""
    if not os.path.exists(src):
        pytest.skip("reference test sources not present")
    from poisson_solver_gb300 import _lib
    exe = tmp_path / prog
    cmd = ["g++", "-std=c++11", "-O1", "-w", "-I", os.path.join(ROOT, "include"), "-I",
           os.path.join(ROOT, "oracle", "mpi_stub"), src, "-o", str(exe), _lib.lib_path(),
           f"-Wl,-rpath,{os.path.dirname(_lib.lib_path())}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_build_is_in_tree(native):
    from poisson_solver_gb300 import _lib
    assert os.path.dirname(_lib.lib_path()).startswith(ROOT)
    assert shutil.which("nvcc") or os.path.exists("/usr/local/cuda/bin/nvcc")
