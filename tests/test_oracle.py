"""The CPU oracle against every known-answer fixture of the reference's own
test suite for this path (test/test_mesh.jl, test_deposition.jl,
test_solvers.jl, test_interpolation.jl, analytical_test.jl) and against
analytic known answers.  CPU only."""
import math

import numpy as np
import pytest

import oracle as O


# ------------------------------------------------------------ test_mesh.jl
def test_particle_ctor_bounds():  # test/test_mesh.jl:8-34
    px, py, pz = [-1.0, 1.0], [-2.0, 2.0], [-3.0, 3.0]
    m = O.mesh_auto((10, 20, 30), px, py, pz)
    assert m.rho.shape == (10, 20, 30) and m.efield.shape == (10, 20, 30, 3)
    for d, p in enumerate((px, py, pz)):
        assert m.min_bounds[d] < min(p) and m.max_bounds[d] > max(p)
        assert m.delta[d] == pytest.approx((m.max_bounds[d] - m.min_bounds[d]) / (m.grid_size[d] - 1))


def test_manual_ctor():  # test_mesh.jl:37-53
    m = O.mesh_manual((10, 20, 30), (-1.0, -2.0, -3.0), (1.0, 2.0, 3.0))
    assert m.min_bounds == (-1.0, -2.0, -3.0) and m.max_bounds == (1.0, 2.0, 3.0)
    assert m.delta == pytest.approx((2 / 9, 4 / 19, 6 / 29))


def test_validation():  # test_mesh.jl:76-94
    for g in [(0, 2, 2), (2, 0, 2), (2, 2, 0), (1, 2, 2), (2, 1, 2), (2, 2, 1)]:
        with pytest.raises(ValueError):
            O.mesh_auto(g, [0.0], [0.0], [0.0])
    with pytest.raises(ValueError):
        O.mesh_auto((2, 2, 2), [], [], [])
    with pytest.raises(ValueError):
        O.mesh_auto((4, 4, 4), [0.0, 1.0], [0.0], [0.0])
    with pytest.raises(ValueError):
        O.mesh_manual((2, 2, 2), (0, 0, 0), (0, 0, 0))
    with pytest.raises(ValueError):
        O.mesh_manual((2, 2, 2), (1, 1, 1), (0, 0, 0))


def test_physics_params():  # test_mesh.jl:97-108
    m = O.mesh_auto((5, 5, 5), [0.0], [0.0], [0.0], gamma=2.0, total_charge=1.0)
    assert m.gamma == 2.0 and m.total_charge == 1.0
    # single particle: span 0 -> delta patched to 1e-6 (mesh.jl:145-149)
    assert m.delta == (1e-6, 1e-6, 1e-6) and m.min_bounds == (0.0, 0.0, 0.0)


# ------------------------------------------------------ test_deposition.jl
@pytest.mark.parametrize("case", ["basic", "multi", "grid_point"])
def test_charge_conservation(case):  # test_deposition.jl:21,41,67
    if case == "basic":
        g, px, py, pz, pq = (4, 4, 4), [0.5], [0.5], [0.5], [1.0]
    elif case == "multi":
        g, px, py, pz, pq = (6, 6, 6), [0.2, 0.8], [0.3, 0.7], [0.4, 0.6], [1.0, -1.0]
    else:
        g, px, py, pz, pq = (4, 4, 4), [0.0], [0.0], [0.0], [1.0]
    m = O.mesh_auto(g, px, py, pz)
    O.deposit(m, px, py, pz, pq)
    assert abs(m.rho.sum() - sum(pq)) < 1e-10
    if case == "multi":
        assert (m.rho > 0).any() and (m.rho < 0).any()


def test_accumulate_and_clear():  # test_deposition.jl:67-113
    m = O.mesh_auto((4, 4, 4), [0.5], [0.5], [0.5])
    O.deposit(m, [0.5], [0.5], [0.5], [1.0])
    first = m.rho.sum()
    O.deposit(m, [0.5], [0.5], [0.5], [1.0], clear=False)
    assert abs(m.rho.sum() - 2 * first) < 1e-10
    O.clear_mesh(m)
    assert (m.rho == 0).all()


def test_particle_at_max_bound():  # test_deposition.jl:83-93
    m = O.mesh_auto((4, 4, 4), [0.0], [0.0], [0.0])
    p = [m.max_bounds[0]], [m.max_bounds[1]], [m.max_bounds[2]]
    m2 = O.mesh_auto((4, 4, 4), *p)
    O.deposit(m2, *p, [1.0])
    assert abs(m2.rho.sum() - 1.0) < 1e-10


def test_cic_known_answer():
    """CIC weights at a known position: node values are the products of
    (1-f, f) per axis (deposition.jl:54-74)."""
    m = O.mesh_manual((4, 4, 4), (0.0, 0.0, 0.0), (3.0, 3.0, 3.0))
    O.deposit(m, [1.25], [0.5], [2.75], [2.0])
    w = np.zeros((4, 4, 4))
    for a, wa in ((1, 0.75), (2, 0.25)):
        for b, wb in ((0, 0.5), (1, 0.5)):
            for c, wc in ((2, 0.25), (3, 0.75)):
                w[a, b, c] = 2.0 * wa * wb * wc
    assert np.array_equal(m.rho, w)


# --------------------------------------------------------- test_solvers.jl
def test_solver_point_charge():  # test_solvers.jl:7-30
    m = O.mesh_auto((16, 16, 16), [0.0], [0.0], [0.0], gamma=2.0)
    O.deposit(m, [0.0], [0.0], [0.0], [1.0])
    O.solve(m)
    assert abs(m.rho.sum() - 1.0) < 1e-10
    assert (m.efield != 0).any() and np.isfinite(m.efield).all()


def test_cathode_changes_field():  # test_solvers.jl:33-56
    args = ((16, 16, 16), [0.0], [0.0], [0.01])
    m = O.mesh_auto(*args, gamma=2.0)
    O.deposit(m, [0.0], [0.0], [0.01], [1.0])
    O.solve(m, at_cathode=True)
    f = O.mesh_auto(*args, gamma=2.0)
    O.deposit(f, [0.0], [0.0], [0.01], [1.0])
    O.solve(f)
    assert not np.allclose(m.efield, f.efield)
    assert np.isfinite(m.efield).all()


def test_gamma_changes_field():  # test_solvers.jl:59-78
    out = []
    for gamma in (1.0, 10.0):
        m = O.mesh_auto((8, 8, 8), [0.0], [0.0], [0.0], gamma=gamma)
        O.deposit(m, [0.0], [0.0], [0.0], [1.0])
        O.solve(m)
        out.append(m.efield.copy())
    assert not np.allclose(out[0], out[1])


# ---------------------------------------------------- test_interpolation.jl
def test_interp_basic():  # test_interpolation.jl:7-33
    m = O.mesh_auto((4, 4, 4), [0.5], [0.5], [0.5])
    m.efield[0, 0, 0, 0] = 1.0
    m.efield[1, 0, 0, 0] = 2.0
    m.efield[0, 1, 0, 0] = 3.0
    m.efield[0, 0, 1, 0] = 4.0
    ex, ey, ez = O.interpolate_field(m, [0.5], [0.5], [0.5])
    assert np.isfinite(ex[0]) and abs(ey[0]) < 1e-10 and abs(ez[0]) < 1e-10


def test_interp_computed_field():  # test_interpolation.jl:87-112
    m = O.mesh_auto((8, 8, 8), [0.0], [0.0], [0.0])
    O.deposit(m, [0.0], [0.0], [0.0], [1.0])
    O.solve(m)
    e = O.interpolate_field(m, [0.0], [0.0], [0.0])
    assert all(abs(c[0]) > 1e7 for c in e)


def test_interp_constant_field():  # test_interpolation.jl:115-133
    m = O.mesh_auto((4, 4, 4), [0.0, 1.0], [0.0, 1.0], [0.0, 1.0])
    m.efield[...] = 1.0
    e = O.interpolate_field(m, [0.0, 1.0], [0.0, 1.0], [0.0, 1.0])
    for c in e:
        assert np.allclose(c, 1.0)


def test_interp_gradient():  # test_interpolation.jl:36-66, exact for a linear field
    m = O.mesh_auto((4, 4, 4), [0.25, 0.75], [0.25, 0.75], [0.25, 0.75])
    i = np.arange(4)
    m.efield[..., 0] = (i[:, None, None] + 1) * 0.1
    m.efield[..., 1] = (i[None, :, None] + 1) * 0.1
    m.efield[..., 2] = (i[None, None, :] + 1) * 0.1
    e = O.interpolate_field(m, [0.25, 0.75], [0.25, 0.75], [0.25, 0.75])
    (ix, iy, iz), (fx, fy, fz) = O.cic_cells(m, [0.25, 0.75], [0.25, 0.75], [0.25, 0.75])
    assert np.allclose(e[0], (ix + fx + 1) * 0.1, rtol=1e-12)
    assert np.allclose(e[2], (iz + fz + 1) * 0.1, rtol=1e-12)


# ------------------------------------------------------ analytical_test.jl
def _gaussian_mesh(n, grid, seed=123, sigma=1e-3, Q=1e-9):
    rng = np.random.default_rng(seed)
    x, y, z = rng.standard_normal((3, n)) * sigma
    q = np.full(n, Q / n)
    m = O.mesh_auto(grid, x, y, z, total_charge=Q)
    O.deposit(m, x, y, z, q)
    O.solve(m)
    return m


def _on_axis_error(m, Q=1e-9, sigma=1e-3):
    nx, ny, nz = m.grid_size
    zc = np.array([m.min_bounds[2] + k * m.delta[2] for k in range(nz)])
    xi = np.argmin(np.abs([m.min_bounds[0] + i * m.delta[0] for i in range(nx)]))
    yi = np.argmin(np.abs([m.min_bounds[1] + i * m.delta[1] for i in range(ny)]))
    ez = m.efield[xi, yi, :, 2]
    ea = O.gaussian_field(np.zeros(nz), np.zeros(nz), zc, Q, sigma)[2]
    return np.abs(ez - ea).max() / np.abs(ea).max()


def test_analytic_gaussian():  # test/analytical_test.jl:7-52 (1M particles, 32^3, < 10%)
    m = _gaussian_mesh(1_000_000, (32, 32, 32))
    assert _on_axis_error(m) < 0.10


def test_boosted_gaussian():
    """A bunch isotropic in its rest frame, contracted by gamma in the lab:
    the reference's gamma scaling (green_functions.jl:73,76-80) must give
    E_lab(x,y,z) = (gamma Ex', gamma Ey', Ez') of the rest-frame Gaussian
    at (x, y, gamma z)."""
    gamma, sigma, Q, n = 4.0, 1e-3, 1e-9, 400_000
    rng = np.random.default_rng(5)
    x, y, z = rng.standard_normal((3, n)) * sigma
    z = z / gamma
    m = O.mesh_manual((32, 32, 32), (-5 * sigma,) * 2 + (-5 * sigma / gamma,), (5 * sigma,) * 2 + (5 * sigma / gamma,),
                      gamma=gamma)
    O.deposit(m, x, y, z, np.full(n, Q / n))
    O.solve(m)
    k = np.arange(32)
    X = m.min_bounds[0] + k * m.delta[0]
    Z = m.min_bounds[2] + k * m.delta[2]
    # transverse field along x through the centre line and Ez along z
    ex_num = m.efield[:, 15, 15, 0]
    yc, zc = m.min_bounds[1] + 15 * m.delta[1], m.min_bounds[2] + 15 * m.delta[2]
    ex_ana = gamma * O.gaussian_field(X, np.full(32, yc), np.full(32, gamma * zc), Q, sigma)[0]
    ez_num = m.efield[15, 15, :, 2]
    xc = m.min_bounds[0] + 15 * m.delta[0]
    ez_ana = O.gaussian_field(np.full(32, xc), np.full(32, yc), gamma * Z, Q, sigma)[2]
    assert np.abs(ex_num - ex_ana).max() / np.abs(ex_ana).max() < 0.08
    assert np.abs(ez_num - ez_ana).max() / np.abs(ez_ana).max() < 0.08


def _cell_integral(d, h, sub=24):
    """Numerical cubature of x/r^3 over the box centred at d with sides h
    (midpoint rule on sub^3 points, Richardson-extrapolated)."""
    def mid(s):
        g = [d[i] + h[i] * ((np.arange(s) + 0.5) / s - 0.5) for i in range(3)]
        X, Y, Z = np.meshgrid(*g, indexing="ij")
        r = np.sqrt(X * X + Y * Y + Z * Z)
        return (X / r ** 3).sum() * h[0] * h[1] * h[2] / s ** 3
    return (4 * mid(2 * sub) - mid(sub)) / 3


def test_igf_vs_cubature():
    """The 8-point difference of the antiderivative (green_functions.jl:35-38,
    103-112) is the cell integral of x/r^3 scaled by gamma/(dx dy dz)."""
    m = O.mesh_manual((6, 6, 6), (0.0,) * 3, (1.0, 1.3, 0.9), gamma=1.5)
    K = O.linear_green_kernel(m, 1)  # x component, indexed by d + n - 1
    dx, dy, dz = m.delta[0], m.delta[1], m.delta[2] * m.gamma
    for d in [(2, 1, 0), (3, 2, 2), (1, 0, 4), (5, 5, 5)]:
        c = tuple(di + 5 for di in d)
        num = _cell_integral((d[0] * dx, d[1] * dy, d[2] * dz), (dx, dy, dz)) * m.gamma / (dx * dy * dz)
        assert K[c] == pytest.approx(num, rel=2e-5)


def test_image_charge():
    """solve!(at_cathode=true) for a point-like charge equals the free field
    of the charge plus that of an opposite charge mirrored through z=0
    (free_space.jl:19-46), evaluated by the same discretisation."""
    g = (12, 12, 12)
    lo, hi = (-1e-3, -1e-3, 0.5e-3), (1e-3, 1e-3, 2.5e-3)
    p = ([0.1e-3], [-0.2e-3], [1.3e-3])
    m = O.mesh_manual(g, lo, hi)
    O.deposit(m, *p, [1e-12])
    O.solve(m, at_cathode=True)
    # brute force: direct sum of cell-integrated kernels over the image charges
    free = O.mesh_manual(g, lo, hi)
    O.deposit(free, *p, [1e-12])
    O.solve(free)
    img = m.efield - free.efield
    # image field at the mesh nodes = field of -rho placed at -z
    nx, ny, nz = g
    zi = np.array([lo[2] + k * m.delta[2] for k in range(nz)])
    rho = free.rho
    e_img = np.zeros(3)
    node = (6, 6, 6)
    xn = lo[0] + node[0] * m.delta[0]
    yn = lo[1] + node[1] * m.delta[1]
    zn = zi[node[2]]
    for (a, b, c) in zip(*np.nonzero(rho)):
        xs, ys, zs = lo[0] + a * m.delta[0], lo[1] + b * m.delta[1], -zi[c]
        r = np.array([xn - xs, yn - ys, zn - zs])
        e_img += -rho[a, b, c] * O.FPEI * r / np.linalg.norm(r) ** 3
    assert np.allclose(img[node], e_img, rtol=2e-3)


# ------------------------------------------------ beside the kick: Boris push
def test_boris_pure_electric_field_is_exact():
    """A uniform E alone: u(t) = u0 + qm E t / c after any number of steps,
    and the drift matches the exact relativistic motion to the step's order."""
    qm, E, dt = -1.75882001076e11, 2.0e6, 1e-12
    st = [np.zeros(1) for _ in range(6)]
    for _ in range(100):
        st = list(O.boris_push(*st, np.zeros(1), np.zeros(1), np.full(1, E), np.zeros(1), np.zeros(1), dt, qm))
    assert np.isclose(st[5][0], qm * E * 100 * dt / O.CLIGHT, rtol=1e-12)


def test_boris_pure_magnetic_field_rotates():
    """B alone conserves |u| and rotates u about B by the Boris angle
    2 atan(w dt / 2) per step, w = qm B / gamma the relativistic cyclotron
    frequency (du/dt = w u x B/|B|)."""
    qm, B, dt = -1.75882001076e11, 0.01, 1e-13
    u0 = 0.5
    st = [np.zeros(1), np.zeros(1), np.zeros(1), np.full(1, u0), np.zeros(1), np.zeros(1)]
    z1 = np.zeros(1)
    n = 2000
    for _ in range(n):
        st = list(O.boris_push(*st, z1, z1, z1, z1, np.full(1, B), dt, qm))
    ux, uy, uz = st[3][0], st[4][0], st[5][0]
    assert np.isclose(np.sqrt(ux * ux + uy * uy + uz * uz), u0, rtol=1e-13)
    w = qm * B / np.sqrt(1 + u0 * u0)
    # B along y: dux/dt = -w uz, duz/dt = w ux
    assert np.isclose(np.arctan2(uz, ux), n * 2 * np.arctan(w * dt / 2), rtol=1e-9)


def test_track_conserves_charge_centroid_momentum():
    """Internal forces only: the bunch's total momentum (charge-weighted,
    equal weights) stays near zero while the bunch expands."""
    rng = np.random.default_rng(4)
    n = 20_000
    x, y, z = rng.standard_normal((3, n)) * 1e-3
    zeros = np.zeros(n)
    q = np.full(n, -1e-12 / n)
    st = O.track((16, 16, 16), x, y, z, zeros, zeros, zeros, q, 1e-11, -1.75882001076e11, 5)
    r0 = np.sqrt(np.mean(x * x + y * y + z * z))
    r1 = np.sqrt(np.mean(st[0] ** 2 + st[1] ** 2 + st[2] ** 2))
    assert r1 > r0  # a negative bunch of electrons expands
    p = np.array([st[3].sum(), st[4].sum(), st[5].sum()])
    assert np.abs(p).max() < 1e-3 * np.abs(st[3]).sum()


# ------------------------------------------------ scalar potential
def test_potential_antiderivative_is_one_over_r():
    """The 8-point difference of potential_green_function over a cell equals
    the cell integral of 1/r (midpoint-refined cubature, 2e-5)."""
    h = 0.1
    for c in ((0.35, 0.2, -0.45), (1.0, 0.7, 0.3), (0.06, 0.07, 0.6)):
        lo = np.array(c) - h / 2
        hi = np.array(c) + h / 2
        F = O.potential_green_function
        val = 0.0
        for a in (0, 1):
            for b in (0, 1):
                for e in (0, 1):
                    sgn = (-1) ** (3 - a - b - e)
                    val += sgn * F(*(lo + np.array([a, b, e]) * h))
        m = 40
        t = (np.arange(m) + 0.5) / m * h
        X, Y, Z = np.meshgrid(lo[0] + t, lo[1] + t, lo[2] + t, indexing="ij")
        ref = np.sum(1 / np.sqrt(X * X + Y * Y + Z * Z)) * (h / m) ** 3
        assert abs(val - ref) < 2e-5 * abs(ref)


def test_potential_of_a_gaussian_bunch():
    """solve_potential of a Gaussian bunch against the analytic potential on
    the z axis (the reference's analytical_test bound, 10 %), and E = -grad phi
    against the field solve (central differences, 3 %)."""
    m = _gaussian_mesh(1_000_000, (32, 32, 32))
    phi = O.solve_potential(m)
    nx, ny, nz = m.grid_size
    zc = np.array([m.min_bounds[2] + k * m.delta[2] for k in range(nz)])
    xi = int(np.argmin(np.abs([m.min_bounds[0] + i * m.delta[0] for i in range(nx)])))
    yi = int(np.argmin(np.abs([m.min_bounds[1] + i * m.delta[1] for i in range(ny)])))
    xc, yc = m.min_bounds[0] + xi * m.delta[0], m.min_bounds[1] + yi * m.delta[1]
    pa = O.gaussian_potential(np.full(nz, xc), np.full(nz, yc), zc, 1e-9, 1e-3)
    assert np.abs(phi[xi, yi, :] - pa).max() / np.abs(pa).max() < 0.10
    ez = -(phi[xi, yi, 2:] - phi[xi, yi, :-2]) / (2 * m.delta[2])
    ref = m.efield[xi, yi, 1:-1, 2]
    assert np.abs(ez - ref).max() / np.abs(ref).max() < 0.03
