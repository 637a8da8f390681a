"""The N > 1 (replicas) aggregation of bench.py on CPU: two gloo ranks."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, out):
    import torch.distributed as dist

    from water_simulation_gb300 import replicas

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    # rank r pretends to have taken (10 + r) ms for 1000 * (r + 1) particle-steps
    out[rank] = replicas.throughput(10.0 + rank, 1000.0 * (rank + 1), world)
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_throughput_uses_max_time_and_total_work():
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
        expected = (1000.0 + 2000.0) / (11.0e-3)
        assert out[0] == pytest.approx(expected)
        assert out[1] == pytest.approx(expected)


def test_single_rank_is_local():
    from water_simulation_gb300 import replicas

    assert replicas.throughput(2.0, 100.0, 1) == pytest.approx(50000.0)
