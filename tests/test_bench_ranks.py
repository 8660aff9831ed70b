"""The multi-GPU path of bench.py is replicas only: every rank runs its own batch
and only the timing is combined (the slowest rank's device time, the moves of
all ranks).  Checked with two gloo ranks on the CPU."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    torch.distributed.init_process_group("gloo", rank=rank, world_size=world)
    dev_s = [0.5, 0.8][rank]        # seconds of device time of each rank's segment
    moves = [1000, 3000][rank]
    t, m = bench.combine_ranks(torch, dev_s, moves, "cpu", world)
    out.put((rank, t, m))
    torch.distributed.destroy_process_group()


def test_combine_ranks_two_gloo_ranks():
    ctx = torch.multiprocessing.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    for p in ps:
        p.join(120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(2))
    for _, t, m in res:
        assert t == 0.8 and m == 4000.0   # max over ranks, sum of moves
    import bench
    assert bench.combine_ranks(torch, 0.25, 7, "cpu", 1) == (0.25, 7.0)
