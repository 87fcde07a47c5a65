"""The multi-GPU form is replicas only (one independent cloud per rank, no
collective on the data path); the only exchange is the timing: the job's time
is the slowest rank's.  Checked here with two gloo ranks on the CPU."""
import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, values, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    out[rank] = bench.max_over_ranks(values[rank], "cpu")
    dist.barrier()
    dist.destroy_process_group()


def test_max_over_two_gloo_ranks():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    manager = ctx.Manager()
    out = manager.dict()
    values = [412.5, 388.25]
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, values, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    assert out[0] == out[1] == max(values)


def test_max_over_ranks_alone():
    import bench
    assert bench.max_over_ranks(3.5, "cpu") == 3.5
