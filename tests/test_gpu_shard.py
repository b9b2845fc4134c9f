"""The single-bunch sharded kick through the library: one rank (the same
field as sc.kick, and global_bounds equal to the particle constructor's
bounds) and two gloo ranks sharing the one GPU."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_kick_sharded_single_rank_equals_kick(sc, cuda):
    import torch

    from spacecharge_gb300.shard import global_bounds, kick_sharded

    rng = np.random.default_rng(2)
    n = 100_000
    x, y, z = (torch.from_numpy(a).cuda() for a in rng.standard_normal((3, n)) * 1e-3)
    q = torch.full((n,), 1e-9 / n, dtype=torch.float64, device="cuda")
    grid = (20, 24, 28)
    lo, hi = global_bounds(grid, x, y, z)
    ref = sc.Mesh3D(grid, x, y, z, precision="fp64")
    assert lo == tuple(ref.min_bounds) and hi == tuple(ref.max_bounds)
    m = sc.Mesh3D(grid, lo, hi, precision="fp64")
    e = kick_sharded(m, x, y, z, q)
    r = sc.kick(ref, x, y, z, q)
    for a, b in zip(e, r):
        assert (a - b).abs().max() <= 1e-10 * b.abs().max()


def _two_rank_worker(rank, world, port, out):
    import os
    import sys

    import torch
    import torch.distributed as dist

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    for p in (root, os.path.join(root, "spacecharge.jl_gb300", "python")):
        if p not in sys.path:
            sys.path.insert(0, p)
    import spacecharge_gb300 as sc
    from spacecharge_gb300.shard import global_bounds, kick_sharded

    sc.load()
    torch.cuda.set_device(0)
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        rng = np.random.default_rng(5)
        n = 60_000
        xyz = rng.standard_normal((3, n)) * np.array([[1e-3], [0.8e-3], [0.3e-3]])
        mine = slice(rank, None, world)
        x, y, z = (torch.from_numpy(np.ascontiguousarray(a[mine])).cuda() for a in xyz)
        qq = torch.full((x.numel(),), 1e-9 / n, dtype=torch.float64, device="cuda")
        grid = (20, 24, 28)
        lo, hi = global_bounds(grid, x, y, z)
        m = sc.Mesh3D(grid, lo, hi, precision="fp64", gamma=3.0)
        e = kick_sharded(m, x, y, z, qq)
        out.put((rank, lo, hi, [t.cpu().numpy() for t in e]))
    finally:
        dist.destroy_process_group()


def test_kick_sharded_two_ranks_through_the_library(sc, cuda):
    """Two gloo ranks, each a process with its own context on the one GPU,
    each holding half of one bunch: global_bounds gives both the whole
    bunch's constructor bounds, and kick_sharded (the library's deposit, a
    gloo all-reduce of rho on the host, the library's solve and gather)
    gives each rank's particles the field sc.kick gives the whole bunch, in
    FP64 to 1e-10.  No kernel waits on another rank: the only exchange is
    the host-side all-reduce between launches."""
    import socket

    import torch
    import torch.multiprocessing as mp

    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_two_rank_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=300) for _ in range(2))
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    rng = np.random.default_rng(5)
    n = 60_000
    xyz = rng.standard_normal((3, n)) * np.array([[1e-3], [0.8e-3], [0.3e-3]])
    x, y, z = (torch.from_numpy(a).cuda() for a in xyz)
    q_ = torch.full((n,), 1e-9 / n, dtype=torch.float64, device="cuda")
    ref_mesh = sc.Mesh3D((20, 24, 28), x, y, z, precision="fp64", gamma=3.0)
    ref = [t.cpu().numpy() for t in sc.kick(ref_mesh, x, y, z, q_)]
    for rank, lo, hi, e in got:
        assert lo == tuple(ref_mesh.min_bounds) and hi == tuple(ref_mesh.max_bounds)
        for c in range(3):
            want = ref[c][rank::2]
            assert np.abs(e[c] - want).max() <= 1e-10 * np.abs(ref[c]).max()
