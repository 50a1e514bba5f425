"""ps_autotune: per-pass kernel family, lines per CTA and (FP32, run-time
kernels) plan variant picked by timing.

Tuning runs on zero-filled scratch buffers, so it must leave pushed fields and
results alone; a tuned solve must agree with the default one to FP32
rounding (other families, line counts and plans only reorder rounding), and
in FP64 (run-time kernels only, default plans, whose per-line arithmetic does
not depend on the line count) bit for bit. Tuned choices go to the cache file
and are reused by a new handle of the same configuration; a cache line
without the plan-variant field reads as the default plan.
"""
import os
import subprocess
import sys

import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu

FAMILIES = {"runtime", "p2", "wide", "tmem", "tma"}


def _solver(psg, nc, bc, precision, curl=True):
    ps = psg.PoissonSolver()
    ps.setup3d(nc, bc, tuple(2.0 / n for n in nc), 2)
    ps.set_return_curl(curl)
    ps.set_precision(precision)
    return ps


def _run(ps, B, nc):
    ps.push(*B)
    ps.solve3d()
    shape = (nc[2], nc[1], nc[0])
    A = [np.empty(shape) for _ in range(3)]
    ps.pull(*A)
    return A


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_autotune_keeps_results_and_persists(native, tmp_path, monkeypatch, precision):
    cache = tmp_path / "tune.txt"
    monkeypatch.setenv("PS_TUNE_CACHE", str(cache))
    nc, bc = (128, 96, 128), (0, 0, 0)
    rng = np.random.default_rng(1)
    B = [rng.standard_normal((nc[2], nc[1], nc[0])) for _ in range(3)]
    ps = _solver(native, nc, bc, precision)
    default_cfg = ps.pass_config(7)
    A0 = _run(ps, B, nc)
    ps.autotune(7)
    tuned = ps.pass_config(7)
    assert all(f in FAMILIES and b >= 1 for f, b in tuned)
    A1 = _run(ps, B, nc)
    if precision == "fp64":
        for a, b in zip(A0, A1):
            assert np.array_equal(a, b)
    else:
        assert rel_l2(A1, A0) < 1e-6
    # tuning on scratch buffers: the pushed fields are untouched
    A2 = [np.empty_like(a) for a in A1]
    ps.solve3d()
    ps.pull(*A2)
    for a, b in zip(A1, A2):
        assert np.array_equal(a, b)
    ps.close()
    lines = cache.read_text().strip().splitlines()
    assert len(lines) == 5 and all(len(l.split()) == 4 for l in lines)
    # a new handle of the same configuration reads the cache
    ps2 = _solver(native, nc, bc, precision)
    assert ps2.pass_config(7) == tuned
    ps2.close()
    # a cache written without the plan-variant field is read (in a new
    # process: the table is loaded once a process) as the default plan
    old = tmp_path / "old.txt"
    old.write_text("".join(" ".join(l.split()[:3]) + "\n" for l in lines))
    code = ("import poisson_solver_gb300 as p; s = p.PoissonSolver(); "
            f"s.setup3d({nc}, {bc}, {tuple(2.0 / n for n in nc)}, 2); s.set_return_curl(True); "
            f"s.set_precision('{precision}'); print(s.pass_config(7))")
    env = dict(os.environ, PS_TUNE_CACHE=str(old))
    out = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, timeout=300,
                         cwd=os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    assert out.returncode == 0, out.stderr
    assert out.stdout.strip() == str([(f, b) for f, b in tuned])
    ps2 = _solver(native, nc, bc, precision)
    # line overrides bypass the tuned table
    monkeypatch.setenv("PS_LINES_Y", "2")
    assert ps2.pass_config(7)[1][1] <= 2
    monkeypatch.delenv("PS_LINES_Y")
    ps2.close()
    assert default_cfg  # the default configuration was reported before tuning


def test_autotune_without_cache_file(native, monkeypatch):
    monkeypatch.setenv("PS_TUNE_CACHE", "")
    nc = (40, 36, 30)
    ps = _solver(native, nc, (1, 1, 0), "fp32", curl=False)
    ps.set_return_grad(True)
    ps.autotune(1)
    cfg = ps.pass_config(1)
    assert len(cfg) == 5 and all(f in FAMILIES for f, _ in cfg)
    rng = np.random.default_rng(2)
    B = rng.standard_normal((nc[2], nc[1], nc[0]))
    B -= B.mean(axis=(1, 2), keepdims=True)
    ps.push(B)
    ps.solve3d()
    A = [np.empty_like(B) for _ in range(3)]
    ps.pull(*A)
    ref, _ = native.solve(nc, (1, 1, 0), tuple(2.0 / n for n in nc), [B, None, None], 2, grad=True,
                          precision="fp64")
    assert rel_l2(A, ref) < 5e-6
    ps.close()


def test_autotune_rejects_bad_masks(native):
    from poisson_solver_gb300 import PSError
    from poisson_solver_gb300 import _lib as L
    ps = _solver(native, (16, 16, 16), (0, 0, 0), "fp32")
    with pytest.raises(PSError) as e:
        ps.autotune(0)
    assert e.value.status == L.PS_ERR_ARGUMENT
    with pytest.raises(PSError) as e:
        ps.autotune(1)  # curl of a scalar
    assert e.value.status == L.PS_ERR_COMPONENTS
    ps.close()
