"""Multi-rank placement and timing reduction on CPU (gloo, world size 2): the
host logic of `bench.py --gpus N` and of sharded ensembles."""
import os
import socket

import pytest

from mpaso.replicas import reduce_over_ranks, shard


def test_shard_covers_every_item_once_and_balances():
    w = [4096, 65536, 1024, 10242, 40962, 2304, 9216, 36864, 16384, 1024]
    for world in (1, 2, 3, 4, 8):
        parts = [shard(w, world, r) for r in range(world)]
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(len(w)))
        loads = [sum(w[i] for i in p) for p in parts]
        assert max(loads) - min(loads) <= max(w)
    with pytest.raises(ValueError):
        shard(w, 2, 2)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, weights, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        mine = shard(weights, world, rank)
        cells = sum(weights[i] for i in mine)
        ms = 10.0 + rank  # this rank's timed region
        out[rank] = (mine, reduce_over_ranks(ms, "max"), reduce_over_ranks(cells, "sum"))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_agree_on_placement_and_timing():
    import torch.multiprocessing as mp
    weights = [4096, 65536, 1024, 10242, 40962, 2304]
    with mp.Manager() as mgr:
        out = mgr.dict()
        mp.spawn(_worker, args=(2, _free_port(), weights, out), nprocs=2, join=True)
        res = dict(out)
    (a, max_a, sum_a), (b, max_b, sum_b) = res[0], res[1]
    assert sorted(a + b) == list(range(len(weights))) and not set(a) & set(b)
    assert max_a == max_b == 11.0  # the job's time is the slowest rank's
    assert sum_a == sum_b == float(sum(weights))
