"""The multi-process path on CPU: two gloo ranks combine their timings the way
bench.py does under torchrun (units summed, slowest rank's time), and seeded
batch shards differ per rank."""
import os
import socket

import pytest
import torch.multiprocessing as mp

from libheom_gb300 import dist as hd


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    r, w, lr = hd.env()
    units = 1000.0 * (r + 1)
    secs = 2.0 + r            # rank 1 is the slowest
    rate, tmax = hd.job_throughput(units, secs)
    out[r] = (r, w, lr, rate, tmax, hd.shard_seed(2, r))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_throughput_and_shards():
    world = 2
    port = _free_port()
    with mp.Manager() as man:
        out = man.dict()
        mp.spawn(_worker, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    assert set(res) == {0, 1}
    for r in (0, 1):
        rank, w, lr, rate, tmax, seed = res[r]
        assert (rank, w, lr) == (r, 2, r)
        assert tmax == pytest.approx(3.0)
        assert rate == pytest.approx(3000.0 / 3.0)
    assert res[0][5] == 2 and res[1][5] != res[0][5]


def test_single_process_fallback():
    rate, t = hd.job_throughput(500.0, 2.0)
    assert rate == 250.0 and t == 2.0
