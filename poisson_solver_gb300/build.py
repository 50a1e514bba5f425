"""Build the native library libps_gb300.so in-tree with nvcc for sm_103a.

Translation units compile in parallel into poisson_solver_gb300/_build/ and
link into poisson_solver_gb300/libps_gb300.so (CUDA runtime linked
statically). Run ``python -m poisson_solver_gb300.build`` or call build().
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libps_gb300.so")
SOURCES = ["ps_kernels.cu", "ps_kernels_df.cu", "ps_kernels_rader.cu", "ps_kernels_p2.cu", "ps_kernels_wide.cu", "ps_kernels_ztm.cu", "ps_kernels_zq.cu", "ps_kernels_yq.cu", "ps_kernels_xq.cu", "ps_kernels_ztc.cu", "ps_greens.cu", "ps_fields.cu", "ps_solver.cpp", "ps_api.cpp", "ps_batch.cpp", "ps_noalloc.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build poisson_solver_gb300")


def _flags() -> list[str]:
    return ["-O3", "-std=c++17", "-lineinfo", *ARCH, "-Xcompiler", "-fPIC",
            "-I", os.path.join(ROOT, "include"), "-I", CSRC]


def _stamp(paths: list[str]) -> float:
    return max(os.path.getmtime(p) for p in paths)


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile (if anything changed) and return the library path."""
    os.makedirs(BUILD, exist_ok=True)
    cc = nvcc()
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".hpp", ".cuh", ".h"))]
    headers.append(os.path.join(ROOT, "include", "poisson_solver_gb300.h"))
    hstamp = _stamp(headers)
    jobs = []
    objs = []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if force or not os.path.exists(o) or os.path.getmtime(o) < max(os.path.getmtime(s), hstamp):
            jobs.append([cc, *_flags(), "-c", s, "-o", o])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout, r.stderr, file=sys.stderr)

    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            list(ex.map(run, jobs))
    if jobs or not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(o) for o in objs):
        tmp = LIB + ".tmp"
        run([cc, "-shared", *ARCH, "-cudart", "static", "-o", tmp, *objs])
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
