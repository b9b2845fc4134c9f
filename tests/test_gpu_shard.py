"""The single-bunch sharded kick on one GPU (world size 1): the same field
as sc.kick, and global_bounds equal to the particle constructor's bounds."""
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
