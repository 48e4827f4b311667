"""The N > 1 path of bench.py is independent replicas (one domain per rank,
no data-path collective): its only collective is the max over ranks of the
timings. Checked with two gloo ranks on the CPU."""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist

    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    t = bench.max_over_ranks(1.5 + rank, dist, device="cpu")
    out[rank] = (t, bench.replicas_value(1000, 10, world, t))
    dist.destroy_process_group()


def test_max_over_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    out = mgr.dict()
    port = _free_port()
    ps = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
    for p in ps:
        p.start()
    for p in ps:
        p.join(120)
        assert p.exitcode == 0
    assert out[0][0] == out[1][0] == 2.5
    assert out[0][1] == pytest.approx(1000 * 10 * 2 / 2.5 / 1e6)


def test_single_rank_passthrough():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.max_over_ranks(3.25) == 3.25
