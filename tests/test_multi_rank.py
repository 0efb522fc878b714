"""The benchmark's N > 1 path on the host: two ranks over gloo on CPU.

Every rank traces a whole replica of the workload (rays, pairs and rooms are
independent; there is no data-path collective), so the only exchange is the
max-over-ranks of the step times. Each rank here reports its own times; both
must come back with the maximum, and the whole-job rate is N x the units of
one rank over the slowest rank's time.
"""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, ws, port, q):
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        got_ws, got_rank, got_local = bench.dist_env()
        mine = [10.0 + rank, 20.0 - 5.0 * rank, 7.0]
        mx = bench.max_over_ranks(mine, ws, device="cpu")
        q.put((rank, got_ws, got_rank, got_local, mx, bench.aggregate_rate(ws, 1000, mx[0])))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_ranks_reduce_to_the_slowest():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, ws, grank, glocal, mx, rate in res:
        assert (ws, grank, glocal) == (2, rank, rank)
        assert mx == [11.0, 20.0, 7.0]
        assert rate == pytest.approx(2 * 1000 / 11e-3)


def test_one_rank_keeps_its_values():
    import bench
    assert bench.max_over_ranks([3.0, 4.5], 1) == [3.0, 4.5]
    assert bench.aggregate_rate(1, 500, 2.0) == pytest.approx(250000.0)
