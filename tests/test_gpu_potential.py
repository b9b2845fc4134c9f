"""sc_solve_potential (the scalar potential beside the field solve) against
the oracle's restatement, and against -grad(phi) = E.  Mixed and FP64 meshes
run the hand-written pipeline (axes up to 128 nodes); plain64 meshes and
longer axes run the FP64 cuFFT schedule."""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu


def rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return np.abs(a - b).max() / np.abs(b).max()


@pytest.mark.parametrize("prec,tol", [("plain64", 1e-10), ("fp64", 1e-10), ("df32", 1e-10), ("mixed", 1e-5)])
@pytest.mark.parametrize("cath,gamma", [(False, 1.0), (False, 5.0), (True, 1.5)])
def test_potential_matches_oracle(sc, cuda, prec, tol, cath, gamma):
    """df32: an FP64 mesh in double-FP32 mode."""
    rng = np.random.default_rng(3)
    n = 30_000
    x, y, z = rng.standard_normal((3, n)).clip(-4.5, 4.5) * np.array([[1e-3], [1.5e-3], [0.4e-3]])
    if cath:
        z = np.abs(z) + 0.1e-3
    q = np.full(n, 1e-9 / n)
    grid = (16, 12, 20)
    om = O.mesh_auto(grid, x, y, z, gamma=gamma)
    O.deposit(om, x, y, z, q)
    ref = O.solve_potential(om, at_cathode=cath)
    m = sc.Mesh3D(grid, x, y, z, precision="fp64" if prec == "df32" else prec, gamma=gamma)
    if prec == "df32":
        m.set_fp64_arithmetic("df32")
    sc.deposit(m, x, y, z, q)
    phi = sc.solve_potential(m, at_cathode=cath)
    assert tuple(phi.shape) == grid
    assert rel(phi.cpu().numpy(), ref) < tol
    if prec == "df32":  # against FP64 mode on the same deposit
        m.set_fp64_arithmetic("fp64")
        assert rel(phi.cpu().numpy(), sc.solve_potential(m, at_cathode=cath).cpu().numpy()) < 1e-12


def test_minus_grad_phi_is_e(sc, cuda):
    """A Gaussian bunch at gamma = 1: the potential's central differences
    match the solved field in the bunch core to a few percent (the two are
    different discretisations of the same field)."""
    rng = np.random.default_rng(4)
    n = 400_000
    x, y, z = rng.standard_normal((3, n)).clip(-5, 5) * 1e-3
    q = np.full(n, 1e-9 / n)
    m = sc.Mesh3D((32, 32, 32), (-5e-3,) * 3, (5e-3,) * 3, precision="fp64")
    sc.deposit(m, x, y, z, q)
    sc.solve(m)
    phi = sc.solve_potential(m).cpu().numpy()
    E = m.efield.cpu().numpy()
    d = m.delta
    ex = -(phi[2:, 1:-1, 1:-1] - phi[:-2, 1:-1, 1:-1]) / (2 * d[0])
    core = E[8:24, 8:24, 8:24, 0]
    assert np.abs(ex[7:23, 7:23, 7:23] - core).max() < 0.03 * np.abs(core).max()


@pytest.mark.parametrize("prec,tol", [("fp64", 1e-10), ("df32", 1e-10), ("mixed", 1e-5)])
@pytest.mark.parametrize("grid,gamma,cath", [((40, 36, 64), 10.0, False), ((32, 32, 48), 3.0, True),
                                             ((32, 32, 64), 4.0, False), ((32, 32, 64), 4.0, True),
                                             ((12, 10, 150), 2.0, False)])
def test_potential_larger_grids(sc, cuda, prec, tol, grid, gamma, cath):
    """Grids where most cells are far from the origin (the mixed build's
    quadrature), boosted cells, the image, a power-of-two grid (32x32x64:
    in double-FP32 mode the Green transform runs in double-FP32 too), and an
    axis of 150 nodes (a 512-point transform: the cuFFT schedule)."""
    rng = np.random.default_rng(8)
    n = 40_000
    x, y, z = rng.standard_normal((3, n)).clip(-4.5, 4.5) * np.array([[1e-3], [0.8e-3], [0.3e-3]])
    if cath:
        z = np.abs(z) + 0.1e-3
    q = np.full(n, 1e-9 / n)
    om = O.mesh_auto(grid, x, y, z, gamma=gamma)
    O.deposit(om, x, y, z, q)
    ref = O.solve_potential(om, at_cathode=cath)
    m = sc.Mesh3D(grid, x, y, z, precision="fp64" if prec == "df32" else prec, gamma=gamma)
    if prec == "df32":
        m.set_fp64_arithmetic("df32")
    sc.deposit(m, x, y, z, q)
    phi = sc.solve_potential(m, at_cathode=cath)
    assert rel(phi.cpu().numpy(), ref) < tol
    # a second solve reuses the cached potential spectrum
    phi2 = sc.solve_potential(m, at_cathode=cath)
    assert rel(phi2.cpu().numpy(), ref) < tol
    if prec == "df32":  # against FP64 mode (which rebuilds an FP64 spectrum)
        m.set_fp64_arithmetic("fp64")
        assert rel(phi.cpu().numpy(), sc.solve_potential(m, at_cathode=cath).cpu().numpy()) < 1e-12
