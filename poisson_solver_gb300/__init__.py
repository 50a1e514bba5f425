"""GB300-native Green's-function FFT Poisson solver.

Solves lap(A) = -B on 3D unbounded, periodic and mixed unbounded/periodic
domains with hand-written sm_103a CUDA FFT passes behind a C ABI
(include/poisson_solver_gb300.h). This package is the Python front end over
that ABI; it mirrors the reference solver class (PoissonSolver) and builds the
native library in-tree (build.py).
"""
from ._lib import PSError, load  # noqa: F401
from .solver import Partition, PoissonBatch, PoissonSolver, solve, solve2d  # noqa: F401

__all__ = ["PoissonSolver", "PoissonBatch", "Partition", "PSError", "load", "solve", "solve2d"]
