"""Failure path of the bulk-copy z kernel: a bounded wait that runs out.

With PS_TEST_WAIT_TIMEOUT=1 every warp of the kernel first waits on an
mbarrier that nothing arrives at. After the wait limit (1 s of the global
timer) the kernel winds down as after any timed-out wait: it drains the
copies it started, frees its tensor memory and sets the handle's device
status word, and the next synchronising call returns PS_ERR_TIMEOUT. No
fault, trap or hang is involved, and the context stays usable: the next
solve without the probe matches the oracle.
"""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu


def test_timed_out_wait_reports_and_recovers(native, oracle, monkeypatch):
    from poisson_solver_gb300 import PSError
    from poisson_solver_gb300 import _lib as L
    nc, bc = (24, 20, 128), (0, 0, 0)  # Pz = 256
    dx = tuple(2.0 / n for n in nc)
    rng = np.random.default_rng(11)
    B = [rng.standard_normal((nc[2], nc[1], nc[0])) for _ in range(3)]
    ps = native.PoissonSolver()
    ps.setup3d(nc, bc, dx, 2)
    ps.set_return_curl(True)
    ps.set_precision("fp32")
    assert ps.pass_config(7)[2][0] == "tma"
    A = [np.empty_like(b) for b in B]

    monkeypatch.setenv("PS_TEST_WAIT_TIMEOUT", "1")
    ps.push(*B)
    ps.solve3d()
    with pytest.raises(PSError) as e:
        ps.pull(*A)
    assert e.value.status == L.PS_ERR_TIMEOUT

    monkeypatch.delenv("PS_TEST_WAIT_TIMEOUT")
    ps.solve3d()
    ps.pull(*A)  # the status word was cleared by the failed call
    ref, _ = oracle.solve3d(nc, bc, dx, B, 2, curl=True)
    assert rel_l2(A, ref) < 5e-6
    ps.close()
