"""The multi-rank path of bench.py (replicas, no data exchange) on two gloo ranks on the
CPU: every rank gets the slowest rank's time, the whole-job rate counts every replica's
work, and the reference arm runs on rank 0 only."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out):
    import torch.distributed as dist

    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms = bench.max_over_ranks(100.0 + 25.0 * rank, dist, "cpu")
    rate = bench.whole_job_rate(world, 1000.0, ms)
    ref = bench.run_reference(type("A", (), {"qubits": 4, "depth": 1, "seed": 0})()) if rank else None
    out.put((rank, ms, rate, ref))
    dist.destroy_process_group()


def test_two_rank_replicas():
    import multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[1] for r in res] == [125.0, 125.0]  # both ranks see the slowest rank's time
    assert res[0][2] == pytest.approx(2 * 1000.0 / 0.125)
    assert res[1][3] == 0  # the reference arm exits on ranks other than 0 without work
