"""Host-side logic of bench.py: byte accounting and the multi-rank aggregation
(world size 2 over gloo on CPU)."""
import os
import socket

import pytest

import bench


def test_algorithmic_bytes_match_the_published_accounting():
    # 512^3 unbounded, 3 -> 3 curl: 84.98 GB in FP64 working precision, 45.7 GB in FP32
    b64 = sum(bench.algorithmic_bytes((512,) * 3, (1024,) * 3, 3, 3, 16, 8))
    b32 = sum(bench.algorithmic_bytes((512,) * 3, (1024,) * 3, 3, 3, 8, 4))
    assert abs(b64 / 84.98e9 - 1) < 0.01
    assert abs(b32 / 45.7e9 - 1) < 0.01
    # 256^3 vector case: 10.64 GB in FP64
    assert abs(sum(bench.algorithmic_bytes((256,) * 3, (512,) * 3, 3, 3, 16, 8)) / 10.64e9 - 1) < 0.01


def test_nominal_flops_match_the_published_count():
    # 512^3 curl (3 -> 3 components on 1024^3 padded points): 4.8e11 FP64 flops a solve
    assert bench.nominal_flops((1024,) * 3, 3, 3) == pytest.approx(6 * 2.5 * 2 ** 30 * 30)
    assert abs(bench.nominal_flops((1024,) * 3, 3, 3) / 4.8e11 - 1) < 0.01


def test_reference_sample_is_the_workload_source():
    # the CPU legs solve the benchmark's own rings (same seed) on a smaller grid
    a = bench.ring_sample(bench.WORKLOADS["rings512"], 32)
    b = bench.ring_sample(bench.WORKLOADS["rings512"], 32)
    assert len(a) == 3 and a[0].shape == (32, 32, 32)
    assert all((x == y).all() for x, y in zip(a, b))
    assert max(float(abs(x).max()) for x in a) > 0


def test_replica_throughput():
    assert bench.replica_throughput(1e6, 10, 2.0, 4) == pytest.approx(20.0)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank_main(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world), RANK=str(rank),
                      LOCAL_RANK=str(rank))
    w, r, local, pg = bench.dist_setup()
    elapsed = 1.0 + r  # the slower rank sets the job time
    bench.barrier(pg)
    worst = bench.max_over_ranks(pg, elapsed)
    q.put((r, w, worst, bench.replica_throughput(1e6, 5, worst, w)))
    pg.destroy_process_group()


def test_two_rank_aggregation_over_gloo():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(2))
    for r, w, worst, value in res:
        assert w == 2 and worst == 2.0
        assert value == pytest.approx(2 * 1e6 * 5 / 2.0 / 1e6)
