"""The N > 1 path of bench.py on CPU: two gloo ranks (independent replicas)
agree on the slowest rank's time and on the whole-job frames/s."""
import os
import socket

import pytest


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    import sys

    import torch

    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    import bench

    r, w, local = bench.dist_env()
    torch.distributed.init_process_group("gloo", rank=r, world_size=w)
    try:
        mine = 1.5 + rank  # seconds each replica took for its frames
        slowest = bench.slowest_rank_seconds(mine, w, torch.device("cpu"))
        q.put((r, local, slowest, bench.replicas_value(10, w, slowest)))
    finally:
        torch.distributed.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_replica():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    out = sorted(q.get(timeout=10) for _ in range(2))
    assert [o[0] for o in out] == [0, 1] and [o[1] for o in out] == [0, 1]
    for _, _, slowest, value in out:
        assert slowest == pytest.approx(2.5)
        assert value == pytest.approx(10 * 2 / 2.5)
