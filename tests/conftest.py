import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle():
    import __graft_entry__
    __graft_entry__.build_oracle()
    from oracle import oracle as o
    return o


@pytest.fixture(scope="session")
def native():
    """The built native library module (built in-tree if out of date)."""
    from poisson_solver_gb300 import build as b
    b.build()
    import poisson_solver_gb300 as ps
    ps.load()
    return ps


def rel_l2(got, ref):
    """Relative L2 error over a list of component arrays (None entries skipped)."""
    num = den = 0.0
    for g, r in zip(got, ref):
        if r is None:
            assert g is None
            continue
        assert g is not None
        num += float(np.sum((np.asarray(g) - r) ** 2))
        den += float(np.sum(np.asarray(r) ** 2))
    return (num / den) ** 0.5 if den > 0 else num ** 0.5


def golden_cases():
    return sorted(f[:-4] for f in os.listdir(GOLDEN) if f.endswith(".npz"))


def load_golden(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    opts = dict(zip(("grad", "div", "curl", "reproject"), (bool(v) for v in z["options"])))
    if len(z["ncell"]) == 2:  # 2D fixture: no reprojection option
        opts.pop("reproject")
    case = dict(ncell=tuple(int(v) for v in z["ncell"]), bc=tuple(int(v) for v in z["bc"]),
                dx=tuple(float(v) for v in z["dx"]), reg=int(z["reg"]), opts=opts)
    case["B"] = [z["B" + c] if "B" + c in z else None for c in "xyz"]
    case["A"] = [z["A" + c] if "A" + c in z else None for c in "xyz"]
    case["RB"] = [z["RB" + c] if "RB" + c in z else None for c in "xyz"]
    return case
