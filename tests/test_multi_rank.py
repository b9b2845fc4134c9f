"""Host logic of the multi-GPU path on CPU: two gloo ranks shard a batch of
bunches with no data-path collective; the shards are disjoint, complete and
balanced, and a max-over-ranks timing reduction behaves as bench.py uses it."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, counts, q):
    import sys

    sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                                    "spacecharge.jl_gb300", "python"))
    from spacecharge_gb300.shard import shard_bunches

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    mine = shard_bunches(counts, world, rank)
    lst = [None] * world
    dist.all_gather_object(lst, mine)
    t = torch.tensor([float(sum(counts[i] for i in mine))])
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    if rank == 0:
        q.put((lst, float(t.item())))
    dist.destroy_process_group()


@pytest.mark.parametrize("world", [2, 3])
def test_shards_disjoint_complete_balanced(world):
    rng = np.random.default_rng(0)
    counts = [int(v) for v in np.exp(rng.uniform(np.log(1e4), np.log(2e6), 64))]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, counts, q)) for r in range(world)]
    for p in procs:
        p.start()
    lst, maxload = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    allidx = sorted(i for s in lst for i in s)
    assert allidx == list(range(64))
    loads = [sum(counts[i] for i in s) for s in lst]
    assert maxload == max(loads)
    assert max(loads) <= sum(counts) / world + max(counts)  # LPT bound


def test_shard_single_rank_is_everything():
    import sys

    sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                                    "spacecharge.jl_gb300", "python"))
    from spacecharge_gb300.shard import shard_bunches

    assert shard_bunches([5, 1, 9], 1, 0) == [0, 1, 2]
    with pytest.raises(ValueError):
        shard_bunches([1], 2, 2)
