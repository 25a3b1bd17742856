"""bench.py's multi-rank logic on CPU (gloo, two ranks on 127.0.0.1): independent replicas take
the slowest rank's time and count every rank's iterations; under torchrun only rank 0 of the
reference arm prints."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms, value = bench.replica_rate(10.0 * (rank + 1), 100, world, dist, device="cpu")
    out.put((rank, ms, value))
    dist.barrier()
    dist.destroy_process_group()


def test_replicas_take_the_slowest_rank():
    import torch.multiprocessing as mp
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
    for rank, ms, value in res:
        assert ms == 20.0                      # max over ranks
        assert value == pytest.approx(2 * 100 / 0.020)  # both ranks' iterations


def test_single_rank_rate():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.replica_rate(50.0, 10, 1) == (50.0, 200.0)


def test_reference_arm_prints_on_rank_zero_only(capsys):
    sys.path.insert(0, ROOT)
    import bench
    assert bench.reference_arm(None, rank=1) is None
    assert capsys.readouterr().out == ""
