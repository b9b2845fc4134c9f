"""Hand-written adjoint (sc_kick_adjoint) against central finite differences
in FP64 and against torch autograd of the FP64 twin of the oracle.

Tolerances: FP64 adjoint vs FD 1e-6 relative (the map is piecewise
quadratic in each particle's position inside its cell, so central
differences that cross no cell face are exact up to rounding); FP64 adjoint
vs autograd 1e-9; mixed adjoint vs autograd 1e-4 (FP32 pipeline)."""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu


def bunch(n, seed, sig=1e-3):
    rng = np.random.default_rng(seed)
    v = rng.standard_normal((3, n)).clip(-4.5, 4.5) * sig
    return v[0], v[1], v[2]


def loss_and_upstream(n, grid, seed):
    rng = np.random.default_rng(seed)
    g = rng.standard_normal((3, n))
    gg = rng.standard_normal(tuple(grid) + (3,)) * 1e-3
    return g, gg


def rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return np.abs(a - b).max() / np.abs(b).max()


# the second size is the differentiation workload's own autograd check:
# 10,000 particles on a 16^3 mesh
@pytest.mark.parametrize("n,grid", [(2000, (12, 10, 14)), (10000, (16, 16, 16))])
@pytest.mark.parametrize("at_cathode", [False, True])
def test_adjoint_vs_torch_autograd(sc, cuda, at_cathode, n, grid):
    import torch

    from oracle import torch_twin

    x, y, z = bunch(n, 1)
    if at_cathode:
        z = np.abs(z) + 0.3e-3
    q = np.random.default_rng(3).uniform(0.5, 1.5, n) * 1e-12
    lo, hi = (-5e-3, -5e-3, -5e-3 if not at_cathode else 0.1e-3), (5e-3, 5e-3, 5e-3)
    g, gg = loss_and_upstream(n, grid, 4)
    om = O.mesh_manual(grid, lo, hi, gamma=2.0)
    tx, ty, tz, tq = (torch.tensor(v, dtype=torch.float64, requires_grad=True) for v in (x, y, z, q))
    ex, ey, ez, E = torch_twin.kick(om, tx, ty, tz, tq, at_cathode=at_cathode)
    L = (ex * torch.from_numpy(g[0])).sum() + (ey * torch.from_numpy(g[1])).sum() + \
        (ez * torch.from_numpy(g[2])).sum() + (E * torch.from_numpy(gg)).sum()
    L.backward()
    ref = [t.grad.numpy() for t in (tx, ty, tz, tq)]
    for prec, tol in (("fp64", 1e-9), ("mixed", 1e-4)):
        m = sc.Mesh3D(grid, lo, hi, precision=prec, gamma=2.0)
        out = sc.kick_adjoint(m, x, y, z, q, g[0], g[1], g[2], gEgrid=gg, at_cathode=at_cathode)
        for name, a, b in zip("xyzq", out, ref):
            err = rel(a.cpu().numpy(), b)
            assert err < tol, f"{prec} d/d{name}: {err:.3e}"


@pytest.mark.parametrize("grid", [(32, 32, 64), (12, 10, 14)])
def test_adjoint_fp64_df32_mode(sc, cuda, grid):
    """An FP64 mesh in double-FP32 mode gives the FP64 mode's adjoint: its
    forward recompute runs in double-FP32, and its adjoint z pass in FP64 on
    the FP64 Green spectrum, rebuilt where the forward kick left the
    double-FP32 one cached (32x32x64)."""
    n = 5000
    x, y, z = bunch(n, 5)
    q = np.full(n, 1e-9 / n)
    lo, hi = (-5e-3,) * 3, (5e-3,) * 3
    g, gg = loss_and_upstream(n, grid, 6)
    out = {}
    for mode in ("fp64", "df32"):
        m = sc.Mesh3D(grid, lo, hi, precision="fp64", gamma=2.0)
        m.set_fp64_arithmetic(mode)
        sc.kick(m, x, y, z, q)  # leaves this mode's Green spectrum cached
        out[mode] = [t.cpu().numpy() for t in sc.kick_adjoint(m, x, y, z, q, g[0], g[1], g[2], gEgrid=gg)]
    for name, a, b in zip("xyzq", out["df32"], out["fp64"]):
        err = rel(a, b)
        assert err < 1e-11, f"d/d{name}: {err:.3e}"


def test_adjoint_vs_finite_differences(sc, cuda):
    """FP64 central differences of L = sum_i g.E(x_i) + sum_n G.E_n on 32
    random particles whose perturbation stays inside their cell."""
    import torch

    n, grid = 20000, (16, 16, 16)
    x, y, z = bunch(n, 7)
    q = np.full(n, 1e-9 / n)
    lo, hi = (-5e-3,) * 3, (5e-3,) * 3
    g, gg = loss_and_upstream(n, grid, 8)
    m = sc.Mesh3D(grid, lo, hi, precision="fp64")
    dx, dy, dz, dq = (t.cpu().numpy() for t in sc.kick_adjoint(m, x, y, z, q, g[0], g[1], g[2], gEgrid=gg))

    def L(px, py, pz, pq):
        e = sc.kick(m, px, py, pz, pq)
        E = m.efield.double().cpu().numpy()
        return sum(float((e[c] * g[c]).sum()) for c in range(3)) + float((E * gg).sum())

    om = O.mesh_manual(grid, lo, hi)
    _, fr = O.cic_cells(om, x, y, z)
    ok = np.where((np.abs(fr - 0.5) < 0.45).all(axis=0))[0]
    pick = np.random.default_rng(9).choice(ok, 32, replace=False)
    h = 1e-3 * om.delta[0]
    for p in pick:
        for arr, grad in ((x, dx), (y, dy), (z, dz)):
            a0 = arr[p]
            arr[p] = a0 + h
            lp = L(x, y, z, q)
            arr[p] = a0 - h
            lm = L(x, y, z, q)
            arr[p] = a0
            fd = (lp - lm) / (2 * h)
            assert abs(fd - grad[p]) <= 1e-6 * max(abs(fd), np.abs(grad).max() * 1e-3), (p, fd, grad[p])
        hq = 1e-3 * q[p]
        q0 = q[p]
        q[p] = q0 + hq
        lp = L(x, y, z, q)
        q[p] = q0 - hq
        lm = L(x, y, z, q)
        q[p] = q0
        fd = (lp - lm) / (2 * hq)
        assert abs(fd - dq[p]) <= 1e-6 * max(abs(fd), np.abs(dq).max() * 1e-3), (p, fd, dq[p])


def test_kick_autograd_function(sc, cuda):
    """torch.autograd through the library (KickFunction) equals the explicit
    adjoint call."""
    import torch

    n, grid = 3000, (16, 16, 16)
    x, y, z = (torch.tensor(v, device="cuda", requires_grad=True) for v in bunch(n, 11))
    q = torch.full((n,), 1e-12, dtype=torch.float64, device="cuda", requires_grad=True)
    m = sc.Mesh3D(grid, (-5e-3,) * 3, (5e-3,) * 3, precision="mixed")
    ex, ey, ez = sc.kick_autograd(m, x, y, z, q)
    (ez * ez * q).sum().backward()
    ref = sc.kick_adjoint(m, x.detach(), y.detach(), z.detach(), q.detach(), None, None,
                          (2 * ez * q).detach())
    # both calls recompute the FP32 forward (atomic order differs), so compare
    # relative to the largest gradient entry
    for t, r in zip((x, y, z), ref[:3]):
        assert (t.grad - r).abs().max() <= 1e-5 * r.abs().max()
    # q also enters the loss directly: dL/dq = Ez^2 + adjoint term
    rq = ref[3] + (ez * ez).detach()
    assert (q.grad - rq).abs().max() <= 1e-5 * rq.abs().max()
