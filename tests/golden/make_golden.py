"""Write the golden fixtures in this directory from the REFERENCE solver itself.

Runs the unmodified reference C++ (built single-rank by oracle/Makefile into
oracle/_ref/libpsref.so) on seeded inputs and stores inputs and outputs as
compressed .npz files. Needs the reference sources (default /root/reference,
or $PS_REFERENCE_ROOT); the tests only read the committed .npz files.

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle  # noqa: E402

# name, ncell, bc, dx, reg, options, pushed components, zero x-y mean
CASES = [
    ("unb_curl_reg0", (12, 10, 8), (0, 0, 0), (0.1, 0.12, 0.15), 0, dict(curl=True), "xyz", False),
    ("unb_scalar_reg2", (16, 16, 16), (0, 0, 0), (0.125, 0.125, 0.125), 2, dict(), "x", False),
    ("unb_div_reg6_odd", (9, 7, 11), (0, 0, 0), (0.2, 0.2, 0.2), 6, dict(div=True), "xyz", False),
    ("per_curl", (12, 10, 8), (1, 1, 1), (0.1, 0.12, 0.15), 0, dict(curl=True), "xyz", False),
    ("per_grad_reg4_odd", (9, 15, 7), (1, 1, 1), (0.2, 0.1, 0.3), 4, dict(grad=True), "xyz", False),
    ("ppf_curl", (12, 10, 8), (1, 1, 0), (0.1, 0.12, 0.15), 0, dict(curl=True), "xyz", True),
    ("ffp_grad", (12, 10, 8), (0, 0, 1), (0.1, 0.12, 0.15), 0, dict(grad=True), "xyz", False),
    ("unb_curl_reproject_rhs", (10, 12, 8), (0, 0, 0), (0.15, 0.1, 0.12), 2,
     dict(curl=True, reproject=True), "xyz", False),
    ("ffp_none_xz_odd", (13, 11, 5), (0, 0, 1), (0.1, 0.1, 0.2), 0, dict(), "xz", False),
    ("per_none_prime", (11, 13, 17), (1, 1, 1), (0.09, 0.08, 0.07), 2, dict(), "y", False),
]


# 2D (setup2d/solve2d): name, ncell, bc, dx, reg, options, pushed components,
# zero mean. The x-unbounded y-periodic combination has no fixture: the
# reference leaves its 1D line kernel unset there (greens2d.cpp:400).
CASES2D = [
    ("2d_unb_grad_reg4", (12, 10), (0, 0), (0.1, 0.12), 4, dict(grad=True), "x", False),
    ("2d_unb_none_xyz_odd", (9, 13), (0, 0), (0.2, 0.15), 0, dict(), "xyz", False),
    ("2d_per_curl_reg2", (12, 10), (1, 1), (0.1, 0.12), 2, dict(curl=True), "z", True),
    ("2d_xper_div", (10, 14), (1, 0), (0.15, 0.1), 0, dict(div=True), "xy", False),
]


def make_inputs(name, ncell, comps, zero_mean):
    rng = np.random.default_rng(sum(map(ord, name)))
    shape = tuple(reversed(ncell))
    axes = tuple(range(1, len(shape)))
    B = []
    for c in "xyz":
        if c in comps:
            b = rng.standard_normal(shape)
            if zero_mean:
                b -= b.mean(axis=axes if len(shape) == 3 else None, keepdims=True)
            B.append(b)
        else:
            B.append(None)
    return B


def main():
    if not oracle.available("reference"):
        oracle.build(os.environ.get("PS_REFERENCE_ROOT", "/root/reference"))
    for name, ncell, bc, dx, reg, opts, comps, zm in CASES + CASES2D:
        B = make_inputs(name, ncell, comps, zm)
        solve = oracle.solve3d if len(ncell) == 3 else oracle.solve2d
        A, RB = solve(ncell, bc, dx, B, reg, want_rhs=True, kind="reference", **opts)
        out = dict(ncell=np.array(ncell), bc=np.array(bc), dx=np.array(dx), reg=np.array(reg),
                   options=np.array([int(opts.get(k, False)) for k in ("grad", "div", "curl", "reproject")]))
        for i, c in enumerate("xyz"):
            if B[i] is not None:
                out["B" + c] = B[i]
            if A[i] is not None:
                out["A" + c] = A[i]
            if RB[i] is not None:
                out["RB" + c] = RB[i]
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
        print(name, {k: v.shape for k, v in out.items() if k[0] in "AR"})


if __name__ == "__main__":
    main()
