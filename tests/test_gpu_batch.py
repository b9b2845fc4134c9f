"""Batched multi-bunch kicks (sc_batch_kick, graph replay) and the FFT
autotuner."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def bunches(nb, seed):
    rng = np.random.default_rng(seed)
    grids = [(16, 16, 16), (24, 16, 32), (32, 32, 32), (12, 12, 20), (16, 16, 16)]
    out = []
    for i in range(nb):
        n = int(rng.integers(2000, 40000))
        sig = rng.uniform(0.2e-3, 2e-3, 3)
        v = rng.standard_normal((3, n)).clip(-4.5, 4.5) * sig[:, None]
        q = np.full(n, rng.uniform(1e-11, 1e-9) / n)
        out.append((grids[i % len(grids)], float(rng.uniform(1, 50)), v[0], v[1], v[2], q))
    return out


def rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return np.abs(a - b).max() / np.abs(b).max()


def test_batch_matches_single_kicks_and_replays(sc, cuda):
    import torch

    spec = bunches(5, 1)
    meshes = [sc.Mesh3D(g, x, y, z, precision="mixed", gamma=gm) for g, gm, x, y, z, q in spec]
    singles = [sc.Mesh3D(g, x, y, z, precision="mixed", gamma=gm) for g, gm, x, y, z, q in spec]
    dev = [[torch.from_numpy(a).cuda() for a in (x, y, z, q)] for _, _, x, y, z, q in spec]
    b = sc.Batch(meshes, nstreams=3)
    out1 = [tuple(t.clone() for t in o) for o in b.kick(*zip(*dev))]
    assert b.graph_nodes > 0
    ref = [sc.kick(m, *d) for m, d in zip(singles, dev)]
    for o, r in zip(out1, ref):
        for a, c in zip(o, r):
            assert rel(a.cpu().numpy(), c.cpu().numpy()) < 1e-5
    # graph replay after the particles move in place gives the moved fields
    for d in dev:
        d[2].mul_(1.1)
    out2 = b.kick(*zip(*dev))
    ref2 = [sc.kick(m, *d) for m, d in zip(singles, dev)]
    for o, r in zip(out2, ref2):
        for a, c in zip(o, r):
            assert rel(a.cpu().numpy(), c.cpu().numpy()) < 1e-5


def test_batch_cathode_and_eager(sc, cuda):
    import torch

    spec = bunches(3, 2)
    meshes = []
    dev = []
    for g, gm, x, y, z, q in spec:
        z = np.abs(z) + 0.1e-3
        meshes.append(sc.Mesh3D(g, x, y, z, precision="mixed", gamma=gm))
        dev.append([torch.from_numpy(a).cuda() for a in (x, y, z, q)])
    b = sc.Batch(meshes)
    b.set_graph(False)
    out = b.kick(*zip(*dev), at_cathode=True)
    assert b.graph_nodes == 0
    for m, d, o in zip(meshes, dev, out):
        r = sc.kick(m, *d, at_cathode=True)
        for a, c in zip(o, r):
            assert rel(a.cpu().numpy(), c.cpu().numpy()) < 1e-5


@pytest.mark.parametrize("prec", ["mixed", "fp64"])
def test_autotune_choice_keeps_parity(sc, cuda, prec):
    import oracle as O

    n = 20000
    rng = np.random.default_rng(5)
    x, y, z = rng.standard_normal((3, n)).clip(-4.5, 4.5) * 1e-3
    q = np.full(n, 1e-9 / n)
    m = sc.Mesh3D((20, 24, 40), x, y, z, precision=prec, gamma=3.0)
    choice = sc.autotune(m)
    assert choice in (0, 2, 3, 4, 5)
    om = O.mesh_auto((20, 24, 40), x, y, z, gamma=3.0)
    O.deposit(om, x, y, z, q)
    O.solve(om)
    sc.deposit(m, x, y, z, q)
    sc.solve(m)
    tol = 1e-5 if prec == "mixed" else 1e-10
    assert rel(m.efield.double().cpu().numpy(), om.efield) < tol


@pytest.mark.parametrize("cache", [True, False])
def test_kick_graph_replay_matches_eager(sc, cuda, cache):
    """Repeated sc_kick calls with the same arrays replay a captured graph;
    the replay sees particles moved in place and equals an eager kick."""
    import torch

    from spacecharge_gb300 import _lib as L
    import ctypes as C

    (g, gm, x, y, z, q), = bunches(1, 11)
    dev = [torch.from_numpy(a).cuda() for a in (x, y, z, q)]
    m = sc.Mesh3D(g, x, y, z, precision="mixed", gamma=gm)
    m.set_green_cache(cache)
    ref = sc.Mesh3D(g, x, y, z, precision="mixed", gamma=gm)
    ref.set_kick_graph(False)
    out = [torch.empty_like(dev[0]) for _ in range(3)]
    s = torch.cuda.current_stream()

    def kick():
        L.call("sc_kick", m.ptr, *[C.c_void_p(t.data_ptr()) for t in dev], dev[0].numel(), L.SC_F64, 0,
               *[C.c_void_p(t.data_ptr()) for t in out], C.c_void_p(s.cuda_stream))

    n0 = m.launch_count()
    for step in range(4):
        kick()  # eager, then eager + capture, then replays
        e = sc.kick(ref, *dev)
        for a, b in zip(out, e):
            assert rel(a.cpu().numpy(), b.cpu().numpy()) < 1e-5
        dev[0].mul_(1.01)  # move the particles in place
    assert m.launch_count() > n0


@pytest.mark.parametrize("at_cathode", [False, True])
@pytest.mark.parametrize("group_bytes,fused", [(0, False), (2**62, True), (64 << 20, False)])
def test_staged_engine_mixed_members(sc, cuda, at_cathode, group_bytes, fused):
    """The staged engine (one launch per stage over a group of bunches)
    beside the per-bunch streams: dense bunches (vector deposit), sparse
    ones (scalar atomics), a mesh with the Green cache off (its spectrum
    rebuilt inside the graph), and members the stages do not take (an FP64
    mesh, a sorted deposit, Lx != Ly) kicked on the streams.  Every bunch
    equals its own kick, for per-bunch and whole-class groups, fused and
    two-pass forward transforms, eager and replayed, and with the engine
    off."""
    import torch

    rng = np.random.default_rng(21)
    plan = [((16, 16, 16), 40000, "mixed", None), ((32, 32, 32), 2000, "mixed", None),
            ((12, 12, 20), 30000, "mixed", "nocache"), ((16, 16, 16), 10000, "fp64", None),
            ((24, 24, 24), 20000, "mixed", "sorted"), ((24, 16, 32), 15000, "mixed", None),
            ((32, 32, 64), 300000, "mixed", None), ((20, 20, 20), 500, "mixed", None),
            ((16, 16, 16), 5000, "mixed", None)]
    meshes, singles, dev = [], [], []
    for g, n, prec, opt in plan:
        sig = rng.uniform(0.3e-3, 1.5e-3, 3)
        x, y, z = rng.standard_normal((3, n)).clip(-4.5, 4.5) * sig[:, None]
        if at_cathode:
            z = np.abs(z) + 0.1e-3
        q = np.full(n, rng.uniform(1e-11, 1e-9) / n)
        gm = float(rng.uniform(1, 20))
        m = sc.Mesh3D(g, x, y, z, precision=prec, gamma=gm)
        r = sc.Mesh3D(g, x, y, z, precision=prec, gamma=gm)
        if opt == "nocache":
            m.set_green_cache(False)
        if opt == "sorted":
            m.set_kick_mode("sorted")
        meshes.append(m)
        singles.append(r)
        dev.append([torch.from_numpy(a).cuda() for a in (x, y, z, q)])
    b = sc.Batch(meshes, nstreams=3)
    b.set_group_bytes(group_bytes)
    b.set_fused_forward(fused)

    def check(out):
        for r, d, o in zip(singles, dev, out):
            ref = sc.kick(r, *d, at_cathode=at_cathode)
            for a, c in zip(o, ref):
                assert rel(a.cpu().numpy(), c.cpu().numpy()) < 1e-5

    out = [tuple(t.clone() for t in o) for o in b.kick(*zip(*dev), at_cathode=at_cathode)]
    staged, launches = b.staged
    # all but the FP64 mesh, the sorted deposit and the Lx != Ly mesh
    assert staged == 6 and launches >= 6
    check(out)
    for step in range(2):  # replays follow particles moved in place
        for d in dev:
            d[0].mul_(1.02)
        check(b.kick(*zip(*dev), at_cathode=at_cathode))
    assert b.graph_nodes > 0
    b.set_staged(False)
    check(b.kick(*zip(*dev), at_cathode=at_cathode))
    assert b.staged == (0, 0)


def test_batch_autotune_keeps_results(sc, cuda):
    """sc_batch_autotune picks a group budget and forward form; kicks after
    it equal single kicks."""
    import torch

    spec = bunches(6, 4)
    meshes = [sc.Mesh3D(g, x, y, z, precision="mixed", gamma=gm) for g, gm, x, y, z, q in spec]
    dev = [[torch.from_numpy(a).cuda() for a in (x, y, z, q)] for _, _, x, y, z, q in spec]
    b = sc.Batch(meshes)
    gb, fused = b.autotune(*zip(*dev))
    assert gb in (0, 48 << 20, 128 << 20, 512 << 20, 2**63 - 1) and fused in (False, True)
    out = b.kick(*zip(*dev))
    for m, d, o in zip(meshes, dev, out):
        o = [t.clone() for t in o]
        r = sc.kick(m, *d)
        for a, c in zip(o, r):
            assert rel(a.cpu().numpy(), c.cpu().numpy()) < 1e-5
