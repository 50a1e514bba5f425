"""Batched solves (ps_batch_*): many independent problems in one launch per pass.

Every problem of a mixed batch -- odd and prime sizes, all four boundary
families, 1-3 components, none/grad/div/curl -- is checked against the
oracle. In FP64 the batched result must also equal the single-problem solve
bit for bit: both run the same run-time transform kernels, whose per-line
arithmetic does not depend on how many lines a CTA holds.
"""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12
FP32_TOL = 5e-6

# (ncell, bc, components, options)
PROBLEMS = [
    ((12, 10, 8), (0, 0, 0), (0,), dict()),
    ((7, 11, 13), (1, 1, 1), (0, 1, 2), dict(curl=True)),
    ((16, 9, 10), (1, 1, 0), (0, 1, 2), dict(div=True)),
    ((10, 14, 6), (0, 0, 1), (0,), dict(grad=True)),
    ((20, 6, 9), (0, 0, 0), (0, 1, 2), dict(grad=True)),
    ((5, 5, 5), (0, 0, 0), (1, 2), dict()),
    ((24, 16, 12), (0, 0, 0), (0, 1, 2), dict(curl=True)),
    ((9, 13, 11), (1, 1, 1), (2,), dict()),
    ((1, 8, 6), (0, 0, 0), (0,), dict()),
    ((18, 20, 7), (1, 1, 0), (0, 1), dict()),
    ((11, 11, 22), (0, 0, 1), (0, 1, 2), dict(curl=True)),
]


def _fields(nc, comps, seed, zero_mean):
    rng = np.random.default_rng(seed)
    shape = (nc[2], nc[1], nc[0])
    out = []
    for c in range(3):
        if c not in comps:
            out.append(None)
            continue
        f = rng.standard_normal(shape)
        if zero_mean:
            f -= f.mean(axis=(1, 2), keepdims=True)
        out.append(f)
    return out


def _dx(nc):
    return (2.0 / nc[0], 1.7 / nc[1], 2.3 / nc[2])


def _make(psg, precision, seed=0):
    b = psg.PoissonBatch(precision)
    data = []
    for i, (nc, bc, comps, opts) in enumerate(PROBLEMS):
        idx = b.add(nc, bc, _dx(nc), (0, 2, 6)[i % 3])
        assert idx == i
        if opts.get("grad"):
            b.set_return_grad(i, True)
        if opts.get("div"):
            b.set_return_div(i, True)
        if opts.get("curl"):
            b.set_return_curl(i, True)
        B = _fields(nc, comps, 100 * seed + i, zero_mean=bc == (1, 1, 0))
        b.push(i, *B)
        data.append(B)
    return b, data


def _pull(b, i):
    nc = PROBLEMS[i][0]
    shape = (nc[2], nc[1], nc[0])
    A = [np.full(shape, np.nan) for _ in range(3)]
    b.pull(i, *A)
    return [a if not np.isnan(a).all() else None for a in A]


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_batch_vs_oracle(native, oracle, precision):
    b, data = _make(native, precision)
    b.solve()
    tol = FP64_TOL if precision == "fp64" else FP32_TOL
    for i, (nc, bc, comps, opts) in enumerate(PROBLEMS):
        ref, _ = oracle.solve3d(nc, bc, _dx(nc), data[i], (0, 2, 6)[i % 3], **opts)
        got = _pull(b, i)
        assert rel_l2(got, ref) < tol, (i, nc, bc, opts)
    assert b.info(native._lib.PS_BATCH_INFO_LAUNCHES_PER_SOLVE) == 5
    assert b.info(native._lib.PS_BATCH_INFO_POINTS) == sum(np.prod(p[0]) for p in PROBLEMS)
    b.close()


def test_batch_fp64_equals_single_solves(native):
    b, data = _make(native, "fp64", seed=3)
    b.solve()
    for i, (nc, bc, comps, opts) in enumerate(PROBLEMS):
        single, _ = native.solve(nc, bc, _dx(nc), data[i], (0, 2, 6)[i % 3], **opts)
        got = _pull(b, i)
        for g, s in zip(got, single):
            assert (g is None) == (s is None)
            if g is not None:
                assert np.array_equal(g, s), (i, nc, bc, opts)
    b.close()


def test_batch_replay_with_new_data_and_option_change(native, oracle):
    b, data = _make(native, "fp64", seed=5)
    b.solve()
    # same components, new values: the captured graph is replayed
    nc, bc, comps, opts = PROBLEMS[6]
    B2 = _fields(nc, comps, 999, zero_mean=False)
    b.push(6, *B2)
    b.solve()
    ref, _ = oracle.solve3d(nc, bc, _dx(nc), B2, (0, 2, 6)[6 % 3], **opts)
    assert rel_l2(_pull(b, 6), ref) < FP64_TOL
    # untouched problems keep their results
    nc0, bc0, _, opts0 = PROBLEMS[0]
    ref0, _ = oracle.solve3d(nc0, bc0, _dx(nc0), data[0], 0, **opts0)
    assert rel_l2(_pull(b, 0), ref0) < FP64_TOL
    # an option change forces a new capture
    b.set_return_curl(6, False)
    b.solve()
    ref, _ = oracle.solve3d(nc, bc, _dx(nc), B2, (0, 2, 6)[6 % 3])
    assert rel_l2(_pull(b, 6), ref) < FP64_TOL
    b.close()


def test_batch_errors(native):
    from poisson_solver_gb300 import PSError
    from poisson_solver_gb300 import _lib as L
    b = native.PoissonBatch("fp64")
    with pytest.raises(PSError) as e:
        b.solve()
    assert e.value.status == L.PS_ERR_STATE
    b.add((8, 8, 8), (0, 0, 0), (0.1, 0.1, 0.1), 0)
    b.add((6, 6, 6), (1, 1, 1), (0.1, 0.1, 0.1), 0)
    b.push(0, np.ones((8, 8, 8)))
    with pytest.raises(PSError) as e:
        b.solve()  # problem 1 has nothing pushed
    assert e.value.status == L.PS_ERR_STATE
    with pytest.raises(PSError) as e:
        b.set_return_curl(5, True)
    assert e.value.status == L.PS_ERR_ARGUMENT
    b.set_return_curl(0, True)
    b.push(1, np.ones((6, 6, 6)))
    with pytest.raises(PSError) as e:
        b.solve()  # curl of a scalar
    assert e.value.status == L.PS_ERR_COMPONENTS
    b.close()


def test_batch_device_pointers_on_a_stream(native, oracle):
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda:0")
    b = native.PoissonBatch("fp64")
    st = torch.cuda.Stream()
    b.set_stream(st.cuda_stream)
    shapes = [((10, 8, 12), (0, 0, 0)), ((9, 9, 9), (1, 1, 1))]
    fields = []
    for i, (nc, bc) in enumerate(shapes):
        b.add(nc, bc, _dx(nc), 2)
        f = torch.randn((nc[2], nc[1], nc[0]), dtype=torch.float64, device=dev)
        fields.append(f)
        b.push_device(i, f.data_ptr())
    b.solve()
    outs = [torch.empty_like(f) for f in fields]
    for i, o in enumerate(outs):
        b.pull_device(i, o.data_ptr())
    b.synchronize()
    for (nc, bc), f, o in zip(shapes, fields, outs):
        ref, _ = oracle.solve3d(nc, bc, _dx(nc), [f.cpu().numpy(), None, None], 2)
        assert rel_l2([o.cpu().numpy()], [ref[0]]) < FP64_TOL
    b.close()


def test_batch_gaussian_family_equals_single_solves(native):
    """Problems switched to the Gaussian-regularised kernel family solve in
    the batch exactly as alone (FP64), next to problems that keep the
    reference's kernels."""
    b = native.PoissonBatch("fp64")
    data, fam = [], []
    for i, (nc, bc, comps, opts) in enumerate(PROBLEMS[:6]):
        b.add(nc, bc, _dx(nc), (0, 2, 6)[i % 3])
        family = "gaussian" if i % 2 == 0 else "spectral"
        b.set_kernel(i, family, 0.0)
        for k, v in opts.items():
            getattr(b, "set_return_" + k)(i, v)
        B = _fields(nc, comps, 40 + i, zero_mean=bc == (1, 1, 0))
        b.push(i, *B)
        data.append(B)
        fam.append(family)
    b.solve()
    for i, (nc, bc, comps, opts) in enumerate(PROBLEMS[:6]):
        single, _ = native.solve(nc, bc, _dx(nc), data[i], (0, 2, 6)[i % 3], kernel=fam[i], **opts)
        got = _pull(b, i)
        for g, s in zip(got, single):
            assert (g is None) == (s is None)
            if g is not None:
                assert np.array_equal(g, s), (i, nc, bc, opts, fam[i])
    b.close()


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_autotuned_batch_gives_the_same_results(native, precision):
    """ps_batch_autotune picks launch shapes and (FP32) plan variants by
    timing; every line's arithmetic is the same in any shape, so the tuned
    FP64 solve (default plans) equals the untuned one bit for bit and the FP32
    one agrees to rounding, and later solves with new data stay correct."""
    b, data = _make(native, precision)
    b.solve()
    before = [_pull(b, i) for i in range(len(PROBLEMS))]
    b.autotune()
    for t, s, v in b.tuning():
        assert t in (64, 128, 256) and s in (2, 4, 8, 16, 32) and 0 <= v <= 7
        assert precision == "fp32" or v == 0  # FP64 batches keep the default plans
    b.solve()
    after = [_pull(b, i) for i in range(len(PROBLEMS))]
    for x, y in zip(before, after):
        for u, v in zip(x, y):
            assert (u is None) == (v is None)
            if u is not None:
                if precision == "fp64":
                    assert np.array_equal(u, v)
                else:
                    assert np.linalg.norm(u - v) <= 1e-6 * np.linalg.norm(v)
    # new pushed data on the tuned shapes, against single-problem solves
    for i, (nc, bc, comps, opts) in enumerate(PROBLEMS):
        B = _fields(nc, comps, 7000 + i, zero_mean=bc == (1, 1, 0))
        b.push(i, *B)
        data[i] = B
    b.solve()
    tol = FP64_TOL if precision == "fp64" else FP32_TOL
    for i, (nc, bc, comps, opts) in enumerate(PROBLEMS):
        ref, _ = native.solve(nc, bc, _dx(nc), data[i], (0, 2, 6)[i % 3], precision=precision, **opts)
        got = _pull(b, i)
        assert rel_l2(got, ref) < tol


# FP32 problems whose padded lengths the compiled families cover run their
# passes with those kernels (routed), beside the batched run-time launch
ROUTED = [
    ((128, 128, 128), (0, 0, 0), (0, 1, 2), dict(curl=True)),  # padded 256^3: the bulk-copy kernels
    ((64, 64, 64), (1, 1, 1), (0,), dict(grad=True)),          # 64^3 periodic: the length-specialised kernels
    ((32, 64, 32), (0, 0, 1), (0, 1, 2), dict()),              # 64 x 128 x 32: specialised x, y; run-time z
    ((17, 12, 10), (0, 0, 0), (0, 1, 2), dict(curl=True)),     # Bluestein lengths: the batched launch
]


def test_fp32_batch_routes_power_of_two_problems(native, oracle):
    from poisson_solver_gb300 import _lib as L
    b = native.PoissonBatch("fp32")
    for rnd in range(2):  # a second solve with new data goes through a rebuilt graph
        data = []
        for i, (nc, bc, comps, opts) in enumerate(ROUTED):
            if rnd == 0:
                assert b.add(nc, bc, _dx(nc), 2) == i
                for k, v in opts.items():
                    getattr(b, f"set_return_{k}")(i, v)
            B = _fields(nc, comps, 900 + 10 * rnd + i, zero_mean=bc == (1, 1, 1))
            b.push(i, *B)
            data.append(B)
        b.solve()
        assert b.info(L.PS_BATCH_INFO_LAUNCHES_PER_SOLVE) > 5  # routed launches beside the batched ones
        for i, (nc, bc, comps, opts) in enumerate(ROUTED):
            shape = (nc[2], nc[1], nc[0])
            A = [np.full(shape, np.nan) for _ in range(3)]
            b.pull(i, *A)
            single, _ = native.solve(nc, bc, _dx(nc), data[i], 2, precision="fp32", **opts)
            ref, _ = oracle.solve3d(nc, bc, _dx(nc), data[i], 2, **opts)
            for a, s in zip(A, single):
                if s is not None:
                    assert np.array_equal(a, s), f"problem {i}: batched and single solves differ"
            assert rel_l2([a for a, s in zip(A, single) if s is not None], [r for r in ref if r is not None]) < FP32_TOL
    b.close()


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_many_right_hand_sides_share_one_kernel_build(native, oracle, precision):
    """Right-hand sides of one problem are problems added with the same setup:
    they copy the first one's kernel octant instead of building their own
    (PS_BATCH_INFO_KERNEL_BUILDS), and every solution still matches the
    oracle and, in FP64, the single-problem solve bit for bit."""
    psg = native
    nc, bc, reg = (24, 18, 14), (0, 0, 0), 2
    other = ((12, 10, 9), (1, 1, 0))
    b = psg.PoissonBatch(precision)
    setups = [(nc, bc)] * 4 + [other] + [(nc, bc)]
    data = []
    for i, (n, c) in enumerate(setups):
        b.add(n, c, _dx(n), reg)
        b.set_return_curl(i, True)
        B = _fields(n, (0, 1, 2), 500 + i, zero_mean=c == (1, 1, 0))
        b.push(i, *B)
        data.append(B)
    assert b.info(psg._lib.PS_BATCH_INFO_KERNEL_BUILDS) == 2
    b.solve()
    tol = FP64_TOL if precision == "fp64" else FP32_TOL
    for i, (n, c) in enumerate(setups):
        shape = (n[2], n[1], n[0])
        A = [np.empty(shape) for _ in range(3)]
        b.pull(i, *A)
        ref, _ = oracle.solve3d(n, c, _dx(n), data[i], reg, curl=True)
        assert rel_l2(A, ref) < tol, i
        if precision == "fp64":
            single, _ = psg.solve(n, c, _dx(n), data[i], reg, precision="fp64", curl=True)
            for x, y in zip(A, single):
                assert np.array_equal(x, y), i
    # a changed kernel family is built anew and is not shared by later adds
    b.set_kernel(0, "gaussian", 0.0)
    b.add(nc, bc, _dx(nc), reg)
    assert b.info(psg._lib.PS_BATCH_INFO_KERNEL_BUILDS) == 3
    b.close()
