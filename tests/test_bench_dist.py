"""The bench's replica path for --gpus N > 1 (one process per GPU, no data
exchange): world-size-2 gloo ranks on the CPU check the max-over-ranks timing
and the whole-job value."""
import multiprocessing as mp
import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, ws, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws),
                      LOCAL_RANK=str(rank))
    import bench
    dist = bench.dist_init(ws, "gloo")
    ms = bench.reduce_max(dist, 100.0 + 50.0 * rank)  # rank 1 is the slow one
    bench.barrier(dist)
    v = bench.whole_job_value(ws, 1e9, 10, ms)
    q.put((rank, ms, v))
    dist.destroy_process_group()


def test_two_rank_replicas_max_timing():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    res = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[1] for r in res] == [150.0, 150.0]
    # 2 ranks x 10 steps x 1 GB in 150 ms
    assert res[0][2] == pytest.approx(2 * 10 * 1e9 / 0.150 / 1e9)
