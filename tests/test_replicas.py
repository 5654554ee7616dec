"""Multi-GPU is replicas only (every rank renders an independent frame, no data exchange); the
whole-job number is all ranks' points over the slowest rank's time.  Exercised here with two
gloo ranks on the CPU, through the helpers bench.py uses under torchrun."""
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


def _rank(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    ms = 100.0 + 50.0 * rank  # rank 1 is the slower replica
    q.put((rank, bench.slowest_rank_ms(ms), bench.replica_throughput(1e9, ms)))
    dist.barrier()
    dist.destroy_process_group()


def test_replica_aggregation_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    for rank, slowest, gps in got:
        assert slowest == pytest.approx(150.0)
        assert gps == pytest.approx(2 * 1e9 / 0.150 / 1e9)


def test_single_process_is_identity():
    import bench
    assert bench.slowest_rank_ms(12.5) == 12.5
    assert bench.replica_throughput(1e9, 1000.0) == pytest.approx(1.0)
