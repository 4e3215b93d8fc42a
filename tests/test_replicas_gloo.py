"""The multi-GPU path is replicas only (independent MPET instances, no
collective on the data path).  Its host logic — barrier and max-over-ranks
job time — runs here as two gloo ranks on the CPU."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    dist.barrier()
    # rank r pretends its 10 steps took (r + 1) * 100 ms
    value, ms = bench.replica_rate((rank + 1) * 100.0, 10)
    out[rank] = (value, ms)
    dist.destroy_process_group()


def test_replica_rate_takes_the_slowest_rank():
    world = 2
    port = _free_port()
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        procs = [ctx.Process(target=_rank, args=(r, world, port, out)) for r in range(world)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        res = dict(out)
    for r in range(world):
        value, ms = res[r]
        assert ms == pytest.approx(200.0)
        # both replicas' 10 steps in the slowest rank's 0.2 s
        assert value == pytest.approx(2 * 10 / 0.2)


def test_replica_rate_single_process():
    import bench
    value, ms = bench.replica_rate(250.0, 5)
    assert ms == 250.0 and value == pytest.approx(20.0)
