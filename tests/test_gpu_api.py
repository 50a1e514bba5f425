"""C-ABI behaviour on the GPU: errors, state rules, device pointers, streams."""
import ctypes

import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu


def _B(nc, k=3, seed=0):
    rng = np.random.default_rng(seed)
    return [rng.standard_normal((nc[2], nc[1], nc[0])) for _ in range(k)]


def test_error_statuses(native):
    from poisson_solver_gb300 import PSError, _lib
    ps = native.PoissonSolver()
    with pytest.raises(PSError) as e:
        ps.solve3d()
    assert e.value.status == _lib.PS_ERR_STATE
    with pytest.raises(PSError) as e:
        ps.setup3d((8, 8, 8), (1, 0, 0), (0.1,) * 3)
    assert e.value.status == _lib.PS_ERR_BOUNDARY and "z-direction must be the periodic" in e.value.message
    with pytest.raises(PSError) as e:
        ps.setup3d((8, 8, 8), (0, 1, 1), (0.1,) * 3)
    assert e.value.status == _lib.PS_ERR_BOUNDARY and "z-direction must be the unbounded" in e.value.message
    with pytest.raises(PSError) as e:
        ps.setup3d((0, 8, 8), (0, 0, 0), (0.1,) * 3)
    assert e.value.status == _lib.PS_ERR_ARGUMENT
    with pytest.raises(PSError) as e:
        ps.setup3d((8, 8, 8), (0, 0, 0), (0.1, float("nan"), 0.1))
    assert e.value.status == _lib.PS_ERR_ARGUMENT
    with pytest.raises(PSError) as e:
        ps.setup3d((8, 8, 8), (0, 0, 0), (0.1,) * 3, -2)
    assert e.value.status == _lib.PS_ERR_ARGUMENT
    # the largest padded transform is 8192 points: 4097 unbounded cells pad to 8194
    with pytest.raises(PSError) as e:
        ps.setup3d((4097, 4, 4), (0, 0, 0), (0.1,) * 3)
    assert e.value.status == _lib.PS_ERR_UNSUPPORTED
    with pytest.raises(PSError) as e:
        ps.setup2d((4, 8193), (1, 1), (0.1, 0.1))
    assert e.value.status == _lib.PS_ERR_UNSUPPORTED
    with pytest.raises(PSError) as e:
        ps.setup2d((8, 8), (0, 2), (0.1, 0.1))
    assert e.value.status == _lib.PS_ERR_BOUNDARY
    ps.setup2d((8, 8), (0, 0), (0.1, 0.1))
    with pytest.raises(PSError) as e:
        ps.solve3d()  # a 2D handle solves with solve2d
    assert e.value.status == _lib.PS_ERR_STATE
    ps.setup3d((8, 8, 8), (0, 0, 0), (0.1,) * 3)
    with pytest.raises(PSError) as e:
        ps.solve2d()  # and a 3D handle with solve3d
    assert e.value.status == _lib.PS_ERR_STATE
    with pytest.raises(PSError) as e:
        ps.solve3d()
    assert e.value.status == _lib.PS_ERR_STATE
    b = _B((8, 8, 8), 1)[0]
    ps.push(b)
    ps.set_return_curl(True)
    with pytest.raises(PSError) as e:
        ps.solve3d()
    assert e.value.status == _lib.PS_ERR_COMPONENTS and "curl option" in e.value.message
    ps.set_return_curl(False)
    ps.set_return_div(True)
    with pytest.raises(PSError) as e:
        ps.solve3d()
    assert e.value.status == _lib.PS_ERR_COMPONENTS
    ps.set_return_div(False)
    ps.push(None, b, None)
    ps.set_return_grad(True)
    with pytest.raises(PSError) as e:
        ps.solve3d()
    assert e.value.status == _lib.PS_ERR_COMPONENTS and "grad option" in e.value.message
    ps.close()


def test_partition_is_the_whole_grid(native):
    with native.PoissonSolver() as ps:
        ps.setup3d((12, 10, 8), (0, 0, 0), (0.1, 0.2, 0.3))
        assert len(ps.partition) == 1
        p = ps.partition[0]
        assert p.ncell == (12, 10, 8) and p.icell == (0, 0, 0) and p.dx == (0.1, 0.2, 0.3)
        assert ps.padded == (24, 20, 16)


def test_pull_semantics(native, oracle):
    nc, dx = (10, 8, 6), (0.1, 0.1, 0.1)
    B = _B(nc)
    shape = (nc[2], nc[1], nc[0])
    with native.PoissonSolver() as ps:
        ps.setup3d(nc, (0, 0, 0), dx, 2)
        ps.push(B[0])
        ps.solve3d()
        ax, ay = np.full(shape, 7.0), np.full(shape, 7.0)
        ps.pull(ax, ay)
        ref, _ = oracle.solve3d(nc, (0, 0, 0), dx, [B[0], None, None], 2)
        assert rel_l2([ax], [ref[0]]) < 1e-12
        assert np.all(ay == 7.0)  # not produced: untouched
        # a new push replaces the component set
        ps.push(*B)
        ps.set_return_curl(True)
        ps.solve3d()
        A = [np.empty(shape) for _ in range(3)]
        RB = [np.empty(shape) for _ in range(3)]
        ps.pull(*A, *RB)
        ref, rref = oracle.solve3d(nc, (0, 0, 0), dx, B, 2, curl=True, want_rhs=True)
        assert rel_l2(A, ref) < 1e-12
        assert rel_l2(RB, rref) < 1e-12
        # precision can change between solves without a new setup
        ps.set_precision("fp32")
        ps.solve3d()
        ps.pull(*A)
        assert rel_l2(A, ref) < 5e-6


def test_returned_rhs_without_filter_is_the_input(native):
    nc = (8, 6, 4)
    B = _B(nc)
    A, RB = native.solve(nc, (1, 1, 1), (0.1,) * 3, B, 0, want_rhs=True)
    assert all(np.array_equal(r, b) for r, b in zip(RB, B))


def test_device_api_matches_host_api(native):
    torch = pytest.importorskip("torch")
    nc, dx = (24, 20, 16), (0.1, 0.1, 0.1)
    B = _B(nc, seed=5)
    host, _ = native.solve(nc, (0, 0, 0), dx, B, 2, curl=True)
    dev = torch.device("cuda:0")
    Bd = [torch.from_numpy(b).to(dev) for b in B]
    Ad = [torch.empty_like(b) for b in Bd]
    with native.PoissonSolver() as ps:
        ps.setup3d(nc, (0, 0, 0), dx, 2)
        ps.set_return_curl(True)
        s = torch.cuda.Stream()
        ps.set_stream(s.cuda_stream)
        with torch.cuda.stream(s):
            ps.solve3d_device([b.data_ptr() for b in Bd], [a.data_ptr() for a in Ad])
        s.synchronize()
        assert rel_l2([a.cpu().numpy() for a in Ad], host) < 1e-14
        # push_device / pull_device
        ps.push_device(*[b.data_ptr() for b in Bd])
        ps.solve3d()
        A2 = [torch.zeros_like(b) for b in Bd]
        ps.pull_device(*[a.data_ptr() for a in A2])
        assert rel_l2([a.cpu().numpy() for a in A2], host) < 1e-14
        # an output pointer left NULL is not written
        A3 = [torch.full_like(b, 3.0) for b in Bd]
        ps.solve3d_device([b.data_ptr() for b in Bd], [A3[0].data_ptr(), 0, A3[2].data_ptr()])
        ps.synchronize()
        assert bool(torch.all(A3[1] == 3.0))
        assert rel_l2([A3[0].cpu().numpy()], [host[0]]) < 1e-14


def test_repeated_setup_and_many_handles(native, oracle):
    handles = [native.PoissonSolver() for _ in range(3)]
    cases = [((8, 8, 8), (0, 0, 0)), ((12, 6, 10), (1, 1, 1)), ((6, 10, 8), (0, 0, 1))]
    for ps, (nc, bc) in zip(handles, cases):
        ps.setup3d(nc, bc, (0.1, 0.1, 0.1))
    for rounds in range(2):
        for ps, (nc, bc) in zip(handles, cases):
            B = _B(nc, 1, seed=rounds)
            ps.push(B[0])
            ps.solve3d()
            a = np.empty((nc[2], nc[1], nc[0]))
            ps.pull(a)
            ref, _ = oracle.solve3d(nc, bc, (0.1, 0.1, 0.1), [B[0], None, None])
            assert rel_l2([a], [ref[0]]) < 1e-12
    # re-setup one handle to a different grid
    handles[0].setup3d((5, 7, 9), (0, 0, 0), (0.2, 0.2, 0.2), 4)
    B = _B((5, 7, 9), 1)
    handles[0].push(B[0])
    handles[0].solve3d()
    a = np.empty((9, 7, 5))
    handles[0].pull(a)
    ref, _ = oracle.solve3d((5, 7, 9), (0, 0, 0), (0.2, 0.2, 0.2), [B[0], None, None], 4)
    assert rel_l2([a], [ref[0]]) < 1e-12
    for ps in handles:
        ps.close()


def test_concurrent_handles_on_threads(native):
    """Independent handles, each on its own stream and host thread, solving at
    the same time (the multi-instance use of the Fortran API's handle table):
    every result equals the same solve run alone."""
    import threading

    import torch
    nc, dx = (48, 40, 56), (0.04, 0.05, 0.035)
    shape = (nc[2], nc[1], nc[0])
    rng = np.random.default_rng(21)
    cases = [((0, 0, 0), "curl"), ((1, 1, 0), "grad"), ((0, 0, 1), "div")]
    B = [[rng.standard_normal(shape) for _ in range(3)] for _ in cases]

    def make(j):
        bc, opt = cases[j]
        ps = native.PoissonSolver()
        ps.setup3d(nc, bc, dx, 4)
        getattr(ps, f"set_return_{opt}")(True)
        ps.set_precision("fp32" if j % 2 else "fp64")
        return ps

    alone = []
    for j in range(len(cases)):
        ps = make(j)
        ps.push(*B[j])
        ps.solve3d()
        A = [np.zeros(shape) for _ in range(3)]
        ps.pull(*A)
        alone.append(A)
        ps.close()
    handles, streams = [], []
    for j in range(len(cases)):
        ps = make(j)
        s = torch.cuda.Stream()
        ps.set_stream(s.cuda_stream)
        handles.append(ps)
        streams.append(s)
    got = [[[np.zeros(shape) for _ in range(3)] for _ in range(4)] for _ in cases]
    errors = []

    def worker(j):
        try:
            for r in range(4):
                handles[j].push(*B[j])
                handles[j].solve3d()
                handles[j].pull(*got[j][r])
        except Exception as e:
            errors.append(e)

    th = [threading.Thread(target=worker, args=(j,)) for j in range(len(cases))]
    for t in th:
        t.start()
    for t in th:
        t.join()
    assert not errors
    for j in range(len(cases)):
        for r in range(4):
            for c in range(3):
                assert np.array_equal(got[j][r][c], alone[j][c])
    for ps in handles:
        ps.close()


def test_dropin_client_runs(native, tmp_path):
    """The header-only C++ class, compiled into a client shaped like the
    reference's validation programs and extended with the kernel family,
    interleaved arrays and smooth3d, runs on the GPU with every call OK."""
    import os
    import subprocess

    from conftest import ROOT
    from poisson_solver_gb300 import _lib
    from test_abi import DROPIN_CLIENT
    src = tmp_path / "client.cpp"
    src.write_text(DROPIN_CLIENT)
    exe = tmp_path / "client"
    cmd = ["g++", "-std=c++11", "-O1", "-I", os.path.join(ROOT, "include"), "-I", os.path.join(ROOT, "oracle", "mpi_stub"),
           str(src), "-o", str(exe), _lib.lib_path(), f"-Wl,-rpath,{os.path.dirname(_lib.lib_path())}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    run = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert run.returncode == 0, run.stdout + run.stderr
