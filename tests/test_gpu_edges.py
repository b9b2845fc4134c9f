"""Edge cases across the entry points: empty and single-particle calls,
repeated graph replays after a geometry-preserving change of mode, FP32
particles through the host kick and the tracking step."""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu


def test_empty_and_single_particle(sc, cuda):
    m = sc.Mesh3D((8, 8, 8), (0.0, 0.0, 0.0), (1.0, 1.0, 1.0), precision="mixed")
    e = sc.kick(m, np.zeros(0), np.zeros(0), np.zeros(0), np.zeros(0))
    assert all(len(a) == 0 for a in e)
    assert float(m.rho.abs().sum()) == 0.0
    e = sc.kick_host(m, np.zeros(0), np.zeros(0), np.zeros(0), np.zeros(0))
    assert all(len(a) == 0 for a in e)
    # one particle: its own field vanishes by symmetry at the node it sits on
    # and the oracle agrees elsewhere
    x = np.array([0.5])
    om = O.mesh_manual((8, 8, 8), (0.0, 0.0, 0.0), (1.0, 1.0, 1.0))
    O.deposit(om, x, x, x, np.array([1e-12]))
    O.solve(om)
    sc.deposit(m, x, x, x, np.array([1e-12]))
    sc.solve(m)
    E = m.efield.cpu().numpy()
    assert np.abs(E - om.efield).max() <= 1e-5 * np.abs(om.efield).max()


def test_graph_replay_follows_mode_and_cache_changes(sc, cuda):
    import torch

    rng = np.random.default_rng(1)
    n = 50_000
    dev = [torch.from_numpy(a).cuda() for a in rng.standard_normal((3, n)) * 1e-3]
    dev.append(torch.full((n,), 1e-9 / n, dtype=torch.float64, device="cuda"))
    m = sc.Mesh3D((16, 16, 16), dev[0], dev[1], dev[2], precision="mixed")
    ref = sc.Mesh3D((16, 16, 16), dev[0], dev[1], dev[2], precision="mixed")
    ref.set_kick_graph(False)
    want = [t.clone() for t in sc.kick(ref, *dev)]
    for mode, cache in (("vector", True), ("vector", False), ("atomic", True), ("sorted", False), ("vector", True)):
        m.set_kick_mode(mode)
        m.set_green_cache(cache)
        for _ in range(3):  # eager + capture, then replays
            got = sc.kick(m, *dev)
            for a, b in zip(got, want):
                assert (a - b).abs().max() <= 1e-5 * b.abs().max(), (mode, cache)


def test_float32_particles_host_kick_and_track(sc, cuda):
    import torch

    rng = np.random.default_rng(3)
    n = 30_000
    x, y, z = (rng.standard_normal((3, n)) * 1e-3).astype(np.float32)
    q = np.full(n, -1e-12 / n, dtype=np.float32)
    m = sc.Mesh3D((16, 16, 16), x, y, z, precision="mixed")
    d = sc.kick(m, x, y, z, q)
    h = sc.kick_host(m, x, y, z, q)
    for a, b in zip(h, d):
        assert a.dtype == torch.float32 and b.dtype == np.float32
        assert np.abs(a.numpy() - b).max() <= 1e-5 * np.abs(b).max()
    st = [torch.from_numpy(a.copy()).cuda() for a in (x, y, z)] + \
         [torch.zeros(n, dtype=torch.float32, device="cuda") for _ in range(3)]
    sc.track(m, *st, torch.from_numpy(q).cuda(), 1e-11, -1.75882001076e11, steps=3)
    r0 = np.sqrt((x.astype(np.float64) ** 2 + y ** 2 + z ** 2).mean())
    r1 = float(torch.sqrt((st[0].double() ** 2 + st[1].double() ** 2 + st[2].double() ** 2).mean()))
    assert r1 > r0 and np.isfinite(r1)


def test_set_bounds_and_refit_match_fresh_meshes(sc, cuda):
    """A mesh re-bounded in place (manual bounds, then the particle bounds of
    another bunch) kicks bit for bit like a mesh built with those bounds; the
    Green spectra and the kick graph follow the new geometry."""
    import torch

    rng = np.random.default_rng(21)
    n = 40_000
    a = [torch.from_numpy(v).cuda() for v in rng.standard_normal((3, n)) * 1e-3]
    b = [torch.from_numpy(v).cuda() for v in rng.standard_normal((3, n)) * 2e-3]
    q = torch.full((n,), 1e-9 / n, dtype=torch.float64, device="cuda")
    grid = (16, 16, 32)
    m = sc.Mesh3D(grid, a[0], a[1], a[2], precision="mixed")
    m.set_kick_mode("deterministic")
    for _ in range(2):  # eager, then a captured graph for this geometry
        sc.kick(m, *a, q)

    def fresh(*args):
        r = sc.Mesh3D(grid, *args, precision="mixed")
        r.set_kick_mode("deterministic")
        return r

    lo, hi = (-6e-3, -5e-3, -7e-3), (6e-3, 5e-3, 7e-3)
    m.set_bounds(lo, hi)
    for ref in (fresh(lo, hi),):
        assert (m.min_bounds, m.max_bounds, m.delta) == (ref.min_bounds, ref.max_bounds, ref.delta)
        got, want = sc.kick(m, *b, q), sc.kick(ref, *b, q)
        assert all(torch.equal(x, y) for x, y in zip(got, want))
        assert torch.equal(m.efield, ref.efield)
    m.refit(b[0], b[1], b[2])
    ref = fresh(b[0], b[1], b[2])
    assert (m.min_bounds, m.max_bounds, m.delta) == (ref.min_bounds, ref.max_bounds, ref.delta)
    got, want = sc.kick(m, *b, q), sc.kick(ref, *b, q)
    assert all(torch.equal(x, y) for x, y in zip(got, want))
    with pytest.raises(sc.SpaceChargeError, match="strictly greater"):
        m.set_bounds((0.0, 0.0, 0.0), (1.0, 0.0, 1.0))
    assert (m.min_bounds, m.max_bounds) == (ref.min_bounds, ref.max_bounds)


@pytest.mark.parametrize("grid", [(16, 16, 32), (64, 64, 128)])
def test_kick_gather_copy_matches_interpolate_field(sc, cuda, grid):
    """The kick's gather (eager, graph replay and the chunked host kick) and
    interpolate_field on the field the kick left agree bit for bit."""
    import torch

    rng = np.random.default_rng(8)
    n = 200_000
    dev = [torch.from_numpy(v).cuda() for v in rng.standard_normal((3, n)) * 1e-3]
    q = torch.full((n,), 1e-9 / n, dtype=torch.float64, device="cuda")
    m = sc.Mesh3D(grid, dev[0], dev[1], dev[2], precision="mixed")
    for _ in range(2):  # eager, then the captured graph
        got = [t.clone() for t in sc.kick(m, *dev, q)]
        want = sc.interpolate_field(m, *dev)
        assert all(torch.equal(a, b) for a, b in zip(got, want))
    host = sc.kick_host(m, *[t.cpu() for t in dev], q.cpu())
    want = [t.cpu() for t in sc.interpolate_field(m, *dev)]
    assert all(torch.equal(a, b) for a, b in zip(host, want))


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_auto_bounds_extrema_and_non_finite(sc, cuda, dtype):
    """The particle constructor's extrema (an integer order-key reduction on
    the device) equal numpy's, across signs and -0.0, and a NaN of either
    sign or an infinity is rejected, as the reference's bounds would be
    unusable."""
    import torch

    rng = np.random.default_rng(17)
    n = 300_001
    pts = [(rng.standard_normal(n) * s + o).astype(dtype) for s, o in ((1e-3, -2e-3), (5.0, 0.0), (1e-9, 1e-9))]
    pts[1][7] = -0.0
    m = sc.Mesh3D((8, 8, 8), *pts, precision="mixed")
    ref = sc.Mesh3D((8, 8, 8), *[torch.from_numpy(p).cuda() for p in pts], precision="mixed")
    assert (m.min_bounds, m.max_bounds) == (ref.min_bounds, ref.max_bounds)
    om = O.mesh_auto((8, 8, 8), *pts)  # numpy extrema, the reference's FP64 padding
    assert m.min_bounds == tuple(om.min_bounds) and m.max_bounds == tuple(om.max_bounds)
    assert m.delta == tuple(om.delta)
    for bad in (np.nan, -np.nan, np.inf, -np.inf):
        q = [p.copy() for p in pts]
        q[1][n // 2] = bad
        with pytest.raises(sc.SpaceChargeError, match="finite"):
            sc.Mesh3D((8, 8, 8), *q, precision="mixed")


def test_kick_out_argument_replays(sc, cuda):
    """kick(..., out=) writes into the caller's tensors; repeated calls with
    the same tensors go eager, eager + capture, then graph replays, and track
    particles moved in place like a mesh that never replays."""
    import torch

    rng = np.random.default_rng(12)
    n = 50_000
    dev = [torch.from_numpy(v).cuda() for v in rng.standard_normal((3, n)) * 1e-3]
    q = torch.full((n,), 1e-9 / n, dtype=torch.float64, device="cuda")
    m = sc.Mesh3D((16, 16, 16), (-6e-3,) * 3, (6e-3,) * 3, precision="mixed")
    ref = sc.Mesh3D((16, 16, 16), (-6e-3,) * 3, (6e-3,) * 3, precision="mixed")
    ref.set_kick_graph(False)
    out = [torch.empty_like(dev[0]) for _ in range(3)]
    for _ in range(4):
        got = sc.kick(m, *dev, q, out=out)
        assert all(a is b for a, b in zip(got, out))
        want = sc.kick(ref, *dev, q)
        for a, b in zip(got, want):
            assert float((a - b).abs().max()) <= 1e-5 * float(b.abs().max())
        dev[1].mul_(1.02)
    with pytest.raises(sc.SpaceChargeError, match="out must be"):
        sc.kick(m, *dev, q, out=[t.float() for t in out])


def test_meshes_kicked_from_two_host_threads(sc, cuda):
    """Different meshes kicked concurrently from two host threads, each on
    its own stream (graph captures are thread-local), give the results of
    kicking them one after the other."""
    import threading

    import torch

    rng = np.random.default_rng(23)
    n = 100_000
    bunches = []
    for k in range(2):
        dev = [torch.from_numpy(v).cuda() for v in rng.standard_normal((3, n)) * (1e-3 * (k + 1))]
        dev.append(torch.full((n,), 1e-9 / n, dtype=torch.float64, device="cuda"))
        bunches.append(dev)
    meshes = [sc.Mesh3D((32, 32, 32), b[0], b[1], b[2], precision="mixed") for b in bunches]
    for m in meshes:
        m.set_kick_mode("deterministic")
    want = [[t.clone() for t in sc.kick(m, *b)] for m, b in zip(meshes, bunches)]
    outs = [[torch.empty_like(b[0]) for _ in range(3)] for b in bunches]
    errors = []

    def work(k):
        try:
            s = torch.cuda.Stream()
            with torch.cuda.stream(s):
                for _ in range(5):  # eager, capture, replays
                    sc.kick(meshes[k], *bunches[k], out=outs[k])
            s.synchronize()
        except Exception as e:  # reported below
            errors.append(e)

    th = [threading.Thread(target=work, args=(k,)) for k in range(2)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    assert not errors, errors
    for got, ref in zip(outs, want):
        assert all(torch.equal(a, b) for a, b in zip(got, ref))


@pytest.mark.parametrize("grid", [(64, 64, 128), (20, 20, 9), (33, 33, 40), (12, 40, 16), (48, 48, 7)])
def test_fused_forward_pass_matches_separate_passes(sc, cuda, grid):
    """A kick that builds the Green spectra runs the forward x and y passes
    separately (the build runs beside them); a repeated kick with the spectra
    cached runs them as one fused pass per z plane where the plane fits in
    shared memory.  With the deterministic deposit both kicks give the same
    field, bit for bit, when ny is even.  With ny odd the separate x pass
    pairs rows across z planes (two real rows per complex FFT) where the fused
    one pairs the last row of a plane with zeros, so the two differ by FP32
    rounding.  The adjoint's fused passes are covered by its
    finite-difference tests."""
    import torch

    rng = np.random.default_rng(17)
    n = 50_000
    pos = [torch.from_numpy(rng.standard_normal(n) * s).cuda() for s in (1e-3, 1e-3, 2e-3)]
    q = torch.full((n,), 1e-9 / n, dtype=torch.float64, device="cuda")
    m = sc.Mesh3D(grid, *pos, precision="mixed", gamma=3.0)
    m.set_kick_mode("deterministic")
    m.set_kick_graph(False)
    first = [t.clone() for t in sc.kick(m, *pos, q)]
    grid_first = m.efield.clone()
    second = [t.clone() for t in sc.kick(m, *pos, q)]
    if grid[1] % 2 == 0:
        assert torch.equal(m.efield, grid_first)
        for a, b in zip(first, second):
            assert torch.equal(a, b)
    else:
        scale = float(grid_first.abs().max())
        assert float((m.efield - grid_first).abs().max()) <= 1e-6 * scale
        for a, b in zip(first, second):
            assert float((a - b).abs().max()) <= 1e-6 * float(b.abs().max())
