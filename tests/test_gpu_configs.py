"""The benchmark workloads at their full sizes.

  * 1e5-particle isotropic Gaussian, 32^3, FP64: every precision against the
    oracle, and the field against the analytic Gaussian field (the
    reference's analytical_test.jl bound, 10 %).
  * 1e6-particle boosted Gaussian (gamma = 10), 64x64x128: mixed against the
    plain FP64 path, max relative error <= 1e-5 on the mesh and at the
    particles.
  * 4e6-particle flat-top cylinder on a cathode, 128^3, auto bounds: mixed
    and FP64 against the plain FP64 path.
  * 1e6-particle Gaussian, 64^3: the adjoint against FP64 central
    differences on 32 particles (1e-6), and the mixed adjoint against the
    FP64 adjoint.
  * 64 uneven bunches on their own meshes: the graph-replayed batch against
    kicks one bunch at a time.
Sizes the oracle cannot finish in seconds are compared between GPU paths,
each of which is tested against the oracle at smaller sizes elsewhere.
"""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu

EPS0 = 8.8541878128e-12


def relerr(a, b):
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    return np.abs(a - b).max() / np.abs(b).max()


def rmserr(a, b):
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def host(t):
    return t.detach().cpu().numpy().astype(np.float64)


def gaussian(n, sig, seed, cut=5.0):
    rng = np.random.default_rng(seed)
    out = []
    for s in sig:
        v = rng.standard_normal(n)
        bad = np.abs(v) > cut
        while bad.any():
            v[bad] = rng.standard_normal(int(bad.sum()))
            bad = np.abs(v) > cut
        out.append(v * s)
    return out


@pytest.mark.parametrize("prec", ["plain64", "fp64", "mixed"])
def test_isotropic_gaussian_1e5_32cubed(sc, cuda, prec):
    n, sigma, Q = 100_000, 1e-3, 1e-9
    x, y, z = gaussian(n, (sigma,) * 3, 123)
    q = np.full(n, Q / n)
    b = ((-5 * sigma,) * 3, (5 * sigma,) * 3)
    om = O.mesh_manual((32, 32, 32), *b, total_charge=Q)
    oe = O.kick(om, x, y, z, q)
    m = sc.Mesh3D((32, 32, 32), *b, precision=prec, total_charge=Q)
    e = sc.kick(m, x, y, z, q)
    tol = 1e-5 if prec == "mixed" else 1e-10
    assert relerr(host(m.efield), om.efield) < tol
    for a, r in zip(e, oe):
        assert relerr(a, r) < tol
    # analytic field on the z axis through the mesh centre
    k = np.arange(32)
    zc = b[0][2] + k * m.delta[2]
    ez = host(m.efield)[15, 15, :, 2]
    xc, yc = b[0][0] + 15 * m.delta[0], b[0][1] + 15 * m.delta[1]
    ea = O.gaussian_field(np.full(32, xc), np.full(32, yc), zc, Q, sigma)[2]
    assert np.abs(ez - ea).max() / np.abs(ea).max() < 0.10


def test_boosted_gaussian_1e6_mixed_vs_fp64(sc, cuda):
    n = 1_000_000
    sig = (1e-3, 1e-3, 1e-4)
    x, y, z = gaussian(n, sig, 42)
    q = np.full(n, 1e-9 / n)
    b = (tuple(-5 * s for s in sig), tuple(5 * s for s in sig))
    res = {}
    for prec in ("plain64", "mixed"):
        m = sc.Mesh3D((64, 64, 128), *b, precision=prec, gamma=10.0, total_charge=1e-9)
        e = sc.kick(m, x, y, z, q)
        res[prec] = (host(m.efield), [host(t) if hasattr(t, "cpu") else t for t in e])
    assert relerr(res["mixed"][0], res["plain64"][0]) <= 1e-5
    assert rmserr(res["mixed"][0], res["plain64"][0]) <= 1e-5
    for a, r in zip(res["mixed"][1], res["plain64"][1]):
        assert relerr(a, r) <= 1e-5


def flat_top_cylinder(n, seed):
    """Uniform cylinder of radius 1 mm and length 2 mm with a 0.05 mm Gaussian
    edge per transverse axis, z in [0.1, 2.1] mm above the cathode."""
    rng = np.random.default_rng(seed)
    r = 1e-3 * np.sqrt(rng.uniform(0, 1, n))
    th = rng.uniform(0, 2 * np.pi, n)
    x = r * np.cos(th) + rng.normal(0, 0.05e-3, n)
    y = r * np.sin(th) + rng.normal(0, 0.05e-3, n)
    z = rng.uniform(0.1e-3, 2.1e-3, n)
    return x, y, z


def test_cathode_cylinder_4e6_128cubed(sc, cuda):
    import torch

    n = 4_000_000
    x, y, z = (torch.from_numpy(v).cuda() for v in flat_top_cylinder(n, 3))
    q = torch.full((n,), 100e-12 / n, dtype=torch.float64, device="cuda")
    res = {}
    for prec in ("plain64", "fp64", "mixed"):
        m = sc.Mesh3D((128, 128, 128), x, y, z, precision=prec, gamma=1.01, total_charge=100e-12)
        e = sc.kick(m, x, y, z, q, at_cathode=True)
        res[prec] = (host(m.efield), [host(t) for t in e])
        assert m.out_of_range() == 0
        del m
        torch.cuda.empty_cache()
    for prec, tol in (("fp64", 1e-10), ("mixed", 1e-5)):
        assert relerr(res[prec][0], res["plain64"][0]) <= tol, prec
        for a, r in zip(res[prec][1], res["plain64"][1]):
            assert relerr(a, r) <= tol, prec


def test_adjoint_1e6_64cubed(sc, cuda):
    """Loss sum_i q_i Ez_i^2 + eps0/2 sum_n |E_n|^2 dV.  FP64 adjoint against
    FP64 central differences on 32 particles whose perturbation stays inside
    their cell (there the loss is a polynomial in the particle's coordinate
    whose terms beyond the quadratic are ~1e-6 of it, so the differences are
    exact to rounding); the mixed adjoint against the FP64 one."""
    import torch

    n, grid = 1_000_000, (64, 64, 64)
    sigma = 1e-3
    lo, hi = (-5 * sigma,) * 3, (5 * sigma,) * 3
    xyz = [torch.from_numpy(v).cuda() for v in gaussian(n, (sigma,) * 3, 4)]
    q = torch.full((n,), 1e-9 / n, dtype=torch.float64, device="cuda")
    dV = float(np.prod([(hi[d] - lo[d]) / (grid[d] - 1) for d in range(3)]))
    grads = {}
    for prec in ("fp64", "mixed"):
        m = sc.Mesh3D(grid, lo, hi, precision=prec)
        ex, ey, ez = sc.kick(m, *xyz, q)
        gez = 2 * q * ez.double()
        gE = (EPS0 * dV) * m.efield.double()
        grads[prec] = [host(t) for t in sc.kick_adjoint(m, *xyz, q, None, None, gez, gEgrid=gE)]
        if prec == "fp64":
            mesh64 = m
    for a, r in zip(grads["mixed"], grads["fp64"]):
        assert np.abs(a - r).max() <= 1e-4 * np.abs(r).max()
    # bitwise reproducible rho, so the loss differences carry no atomic-order noise
    mesh64.set_kick_mode("deterministic")

    def loss():
        e = sc.kick(mesh64, *xyz, q)
        E = mesh64.efield
        return float((q * e[2] * e[2]).sum() + 0.5 * EPS0 * dV * (E * E).sum())

    om = O.mesh_manual(grid, lo, hi)
    hx = [t.cpu().numpy() for t in xyz]
    _, fr = O.cic_cells(om, *hx)
    # One particle of 1e6 moves the loss by ~1e-10 of itself per 1e-3 cell.
    # Steps of 5 % of a cell keep the FP64 rounding of the loss far below 1e-6
    # of the difference for gradients above 1 % of the largest; smaller ones
    # are held to 1e-6 of that 1 % (the rounding floor of the loss).
    ok = np.where((np.abs(fr - 0.5) < 0.4).all(axis=0))[0]
    pick = np.random.default_rng(9).choice(ok, 32, replace=False)
    h = 0.05 * min(om.delta)
    dx, dy, dz, dq = grads["fp64"]
    for p in pick:
        for c, g in enumerate((dx, dy, dz)):
            a0 = float(xyz[c][p])
            xyz[c][p] = a0 + h
            lp = loss()
            xyz[c][p] = a0 - h
            lm = loss()
            xyz[c][p] = a0
            fd = (lp - lm) / (2 * h)
            assert abs(fd - g[p]) <= 1e-6 * max(abs(fd), np.abs(g).max() * 1e-2), (p, c, fd, g[p])
        q0 = float(q[p])
        hq = 0.05 * q0
        q[p] = q0 + hq
        lp = loss()
        q[p] = q0 - hq
        lm = loss()
        q[p] = q0
        # q also enters the loss directly through q_i Ez_i^2
        fd = (lp - lm) / (2 * hq)
        ez = sc.kick(mesh64, *xyz, q)[2]
        want = dq[p] + float(ez[p]) ** 2
        assert abs(fd - want) <= 1e-6 * max(abs(fd), np.abs(dq).max() * 1e-2), (p, fd, want)


def uneven_bunches(nb, seed):
    """Particle counts log-uniform in [1e4, 2e6], sigma uniform in
    [0.2, 2] mm per axis, gamma uniform in [1, 50], charge uniform in
    [10 pC, 1 nC], grid drawn from {32^3, 64^3, 64x64x128, 128^3}."""
    grids = [(32, 32, 32), (64, 64, 64), (64, 64, 128), (128, 128, 128)]
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(nb):
        n = int(np.exp(rng.uniform(np.log(1e4), np.log(2e6))))
        sig = rng.uniform(0.2e-3, 2e-3, 3)
        gamma = float(rng.uniform(1.0, 50.0))
        qtot = float(rng.uniform(10e-12, 1e-9))
        grid = grids[int(rng.integers(0, len(grids)))]
        v = rng.standard_normal((3, n)) * sig[:, None]
        out.append((grid, gamma, v[0].copy(), v[1].copy(), v[2].copy(), np.full(n, qtot / n)))
    return out


def test_batch_64_uneven_bunches_vs_plain_fp64(sc, cuda):
    """Every bunch of the 64-bunch workload (seed 7: gamma up to 50 and
    sigma_z / sigma_x up to 10, so boosted cells up to ~500 times longer than
    wide), kicked by the mixed-precision batch, against the plain FP64 path
    (the reference algorithm) on the same bounds: max and RMS relative error
    <= 1e-5 on the mesh field and at the particles."""
    import torch

    spec = uneven_bunches(64, 7)
    dev = [[torch.from_numpy(a).cuda() for a in s[2:]] for s in spec]
    meshes = [sc.Mesh3D(g, d[0], d[1], d[2], precision="mixed", gamma=gm) for (g, gm, *_), d in zip(spec, dev)]
    b = sc.Batch(meshes)
    xs, ys, zs, qs = zip(*dev)
    b.kick(xs, ys, zs, qs)
    out = [[host(t) for t in o] for o in b.kick(xs, ys, zs, qs)]
    worst = (0.0, None)
    for i, ((g, gm, *_), m, d, o) in enumerate(zip(spec, meshes, dev, out)):
        emix = host(m.efield)
        mp = sc.Mesh3D(g, d[0], d[1], d[2], precision="plain64", gamma=gm)
        assert mp.delta == m.delta and mp.min_bounds == m.min_bounds
        ref = [host(t) for t in sc.kick(mp, *d)]
        eref = host(mp.efield)
        errs = [relerr(emix, eref), rmserr(emix, eref)]
        for a, r in zip(o, ref):
            errs += [relerr(a, r), rmserr(a, r)]
        cell = gm * m.delta[2] / min(m.delta[0], m.delta[1])
        if max(errs) > worst[0]:
            worst = (max(errs), (i, g, round(gm, 2), round(cell, 1)))
        assert max(errs) <= 1e-5, (i, g, gm, cell, errs)
        del mp
    print("worst bunch vs plain FP64:", worst)


def test_batch_64_uneven_bunches(sc, cuda):
    import torch

    spec = uneven_bunches(64, 7)
    dev = [[torch.from_numpy(a).cuda() for a in s[2:]] for s in spec]
    meshes = [sc.Mesh3D(g, d[0], d[1], d[2], precision="mixed", gamma=gm) for (g, gm, *_), d in zip(spec, dev)]
    b = sc.Batch(meshes)
    xs, ys, zs, qs = zip(*dev)
    b.kick(xs, ys, zs, qs)  # eager run and capture
    out = [[host(t) for t in o] for o in b.kick(xs, ys, zs, qs)]  # graph replay
    assert b.graph_nodes > 0
    for m, d, o in zip(meshes, dev, out):
        ref = sc.kick(m, *d)
        for a, r in zip(o, ref):
            assert relerr(a, host(r)) < 1e-5
