"""sc_track: tracking steps of a bunch in its own field (refit, kick, B from
E, relativistic Boris step) against the oracle's restatement, and a uniform
sphere's Coulomb explosion against its analytic envelope."""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu

QM_E = -1.75882001076e11  # electron charge/mass [C/kg]


def state(n, seed, u_scale=0.0):
    rng = np.random.default_rng(seed)
    x, y, z = rng.standard_normal((3, n)).clip(-4.5, 4.5) * np.array([[1e-3], [1e-3], [0.5e-3]])
    ux, uy, uz = rng.standard_normal((3, n)) * u_scale
    return [x, y, z, ux, uy, uz]


@pytest.mark.parametrize("prec,tol", [("fp64", 1e-9), ("mixed", 2e-5)])
@pytest.mark.parametrize("refit", [True, False])
def test_track_matches_oracle(sc, cuda, prec, tol, refit):
    import torch

    n, grid, steps, dt = 20_000, (16, 16, 20), 4, 2e-11
    st = state(n, 1, u_scale=1e-3)
    q = np.full(n, -2e-12 / n)
    # fixed bounds need room for the bunch to move
    lo = tuple(float(st[d].min()) - 0.5e-3 for d in range(3))
    hi = tuple(float(st[d].max()) + 0.5e-3 for d in range(3))
    m = sc.Mesh3D(grid, st[0], st[1], st[2], precision=prec) if refit else sc.Mesh3D(grid, lo, hi, precision=prec)
    dev = [torch.from_numpy(a.copy()).cuda() for a in st]
    tq = torch.from_numpy(q).cuda()
    sc.track(m, *dev, tq, dt, QM_E, steps=steps, refit=refit)
    if refit:
        ref = O.track(grid, *st, q, dt, QM_E, steps)
    else:
        # fixed bounds: the mesh the library was built with, every step
        om = O.mesh_manual(grid, lo, hi)
        ref = [a.copy() for a in st]
        for _ in range(steps):
            e = O.kick(om, ref[0], ref[1], ref[2], q)
            b = O.magnetic_field(om, e[0], e[1])
            ref = list(O.boris_push(*ref, *e, *b, dt, QM_E))
    got = [t.cpu().numpy() for t in dev]
    for c in range(3):  # displacements and momenta relative to their scale
        d_got, d_ref = got[c] - st[c], ref[c] - st[c]
        assert np.abs(d_got - d_ref).max() <= tol * np.abs(d_ref).max(), c
        assert np.abs(got[3 + c] - ref[3 + c]).max() <= tol * np.abs(ref[3 + c]).max(), c


def test_coulomb_explosion_of_a_uniform_sphere(sc, cuda):
    """An electron sphere of uniform density stays uniform while it expands;
    its edge radius obeys R'' = qm Q / (4 pi eps0 R^2) (non-relativistic here,
    beta < 1e-2).  The RMS radius sqrt(3/5) R of the tracked bunch follows
    the integrated R(t) to 2 % (the mesh smooths the sphere's edge over a
    cell or two) while the sphere grows by a quarter."""
    import torch
    from scipy.integrate import solve_ivp

    n, R0, Q = 400_000, 1e-3, -1e-12
    rng = np.random.default_rng(8)
    v = rng.standard_normal((3, n))
    v *= R0 * rng.uniform(0, 1, n) ** (1 / 3) / np.linalg.norm(v, axis=0)
    dev = [torch.from_numpy(a.copy()).cuda() for a in v] + [torch.zeros(n, dtype=torch.float64, device="cuda")
                                                            for _ in range(3)]
    q = torch.full((n,), Q / n, dtype=torch.float64, device="cuda")
    m = sc.Mesh3D((48, 48, 48), dev[0], dev[1], dev[2], precision="mixed")
    dt, steps = 3e-12, 200
    sc.track(m, *dev, q, dt, QM_E, steps=steps, refit=True)
    r_rms = float(torch.sqrt((dev[0] ** 2 + dev[1] ** 2 + dev[2] ** 2).mean()))
    k = QM_E * Q * O.FPEI

    def rhs(t, s):
        return [s[1], k / s[0] ** 2]

    sol = solve_ivp(rhs, (0, dt * steps), [R0, 0.0], rtol=1e-10, atol=1e-14)
    R = sol.y[0, -1]
    assert R > 1.2 * R0  # the sphere has grown by a fifth or more
    want = np.sqrt(3 / 5) * R
    assert abs(r_rms - want) <= 0.02 * want, (r_rms, want)
    vmax = float(torch.sqrt(dev[3] ** 2 + dev[4] ** 2 + dev[5] ** 2).max())
    assert vmax < 1e-2
