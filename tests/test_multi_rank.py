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


# ------------------------------------------- one bunch split over ranks
def _bunch(n=6000, seed=11):
    rng = np.random.default_rng(seed)
    v = rng.standard_normal((3, n)).clip(-4.5, 4.5) * np.array([[1e-3], [0.8e-3], [0.3e-3]])
    return v[0], v[1], v[2], np.full(n, 1e-9 / n)


class _OracleMesh:
    """Stand-in mesh for the host-logic test: the oracle's mesh with its rho
    exposed as a torch view, as Mesh3D.rho exposes the device array."""

    def __init__(self, grid, lo, hi):
        import oracle as O

        self.om = O.mesh_manual(grid, lo, hi)
        self.rho = torch.from_numpy(self.om.rho)  # x fastest: permute(2, 1, 0) is contiguous


def _sharded_worker(rank, world, port, q):
    import sys

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    sys.path.insert(0, os.path.join(root, "spacecharge.jl_gb300", "python"))
    import oracle as O
    import spacecharge_gb300.mesh as M
    from spacecharge_gb300 import shard

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    x, y, z, qq = _bunch()
    mine = slice(rank, None, world)  # this rank's particles
    grid = (10, 12, 16)
    lo, hi = shard.global_bounds(grid, torch.from_numpy(x[mine]), torch.from_numpy(y[mine]),
                                 torch.from_numpy(z[mine]))
    # the library's deposit/solve/gather replaced by the oracle's (no GPU here)
    M.deposit = lambda m, px, py, pz, pq: O.deposit(m.om, px, py, pz, pq)
    M.solve = lambda m, at_cathode=False: O.solve(m.om, at_cathode=at_cathode)
    M.interpolate_field = lambda m, px, py, pz: O.interpolate_field(m.om, px, py, pz)
    m = _OracleMesh(grid, lo, hi)
    e = shard.kick_sharded(m, x[mine], y[mine], z[mine], qq[mine])
    got = [None] * world
    dist.all_gather_object(got, (rank, lo, hi, [np.asarray(c) for c in e]))
    if rank == 0:
        q.put(got)
    dist.destroy_process_group()


def test_one_bunch_split_over_two_ranks():
    """Two gloo ranks each hold half of one bunch: global_bounds gives both the
    whole bunch's constructor bounds, and kick_sharded (local deposit, rho
    all-reduce, solve, local gather) gives each rank's particles the field of
    the whole bunch."""
    import oracle as O

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_sharded_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = q.get(timeout=180)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    x, y, z, qq = _bunch()
    ref_mesh = O.mesh_auto((10, 12, 16), x, y, z)
    ref = O.kick(ref_mesh, x, y, z, qq)
    for rank, lo, hi, e in got:
        assert np.allclose(lo, ref_mesh.min_bounds, rtol=0, atol=0)
        assert np.allclose(hi, ref_mesh.max_bounds, rtol=0, atol=0)
        for c in range(3):
            want = ref[c][rank::2]
            assert np.abs(e[c] - want).max() <= 1e-12 * np.abs(ref[c]).max()
