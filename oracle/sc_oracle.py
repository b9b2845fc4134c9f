"""FP64 CPU restatement of SpaceCharge.jl's space-charge kick (test oracle).

Every function cites the reference file:line it follows.  Arrays use the
reference's memory layout: rho has shape (nx, ny, nz) and efield (nx, ny, nz, 3),
both Fortran-ordered (x fastest, component-planar), so ``a.ravel(order="F")``
is the flat layout the CUDA library uses for its FP64 plain path.

This module is test infrastructure.  Nothing in the product imports it.
"""
from __future__ import annotations

import math
import os

import numpy as np
import scipy.fft as sfft

__all__ = [
    "CLIGHT", "FPEI", "EPSILON_0", "OMesh", "mesh_auto", "mesh_manual",
    "clear_mesh", "deposit", "field_green_function", "green_function",
    "solve_freespace", "solve", "interpolate_field", "cic_cells",
    "gaussian_field", "kick", "linear_green_kernel", "magnetic_field", "boris_push", "track",
    "potential_green_function", "potential_green", "solve_potential", "gaussian_potential",
]

# src/utils.jl:7-8
CLIGHT = 299792458.0
FPEI = CLIGHT ** 2 * 1.0e-7
# test/analytical_test.jl:9
EPSILON_0 = 8.8541878128e-12

_WORKERS = max(1, os.cpu_count() or 1)


class OMesh:
    """Restates the fields of `Mesh3D` (src/mesh.jl:19-34)."""

    def __init__(self, grid_size, lo, hi, delta, gamma, total_charge, T):
        self.grid_size = tuple(int(g) for g in grid_size)
        self.T = np.dtype(T)
        self.min_bounds = tuple(self.T.type(v) for v in lo)
        self.max_bounds = tuple(self.T.type(v) for v in hi)
        self.delta = tuple(self.T.type(v) for v in delta)
        self.gamma = self.T.type(gamma)
        self.total_charge = self.T.type(total_charge)
        self.rho = np.zeros(self.grid_size, dtype=self.T, order="F")
        self.efield = np.zeros(self.grid_size + (3,), dtype=self.T, order="F")


def _check_grid(grid_size):
    # src/mesh.jl:106-108 and :206-208
    if any(int(g) <= 1 for g in grid_size):
        raise ValueError("All elements of grid_size must be at least 2.")


def mesh_auto(grid_size, px, py, pz, T=np.float64, gamma=1.0, total_charge=0.0):
    """Particle-bounds constructor, src/mesh.jl:95-174 (Float64 arithmetic)."""
    _check_grid(grid_size)
    px, py, pz = (np.asarray(a) for a in (px, py, pz))
    if px.size == 0 or py.size == 0 or pz.size == 0:  # :110-112
        raise ValueError("Particle arrays cannot be empty.")
    if not (px.size == py.size == pz.size):  # :114-116
        raise ValueError("Particle coordinate arrays must have the same length.")
    # :120-122 extrema, then :125-142 in Float64 (the particle eltype promotes)
    mins = [float(a.min()) for a in (px, py, pz)]
    maxs = [float(a.max()) for a in (px, py, pz)]
    n = [int(g) for g in grid_size]
    delta = [(maxs[d] - mins[d]) / (n[d] - 1) for d in range(3)]
    lo = [mins[d] - 1e-6 * delta[d] for d in range(3)]
    hi = [maxs[d] + 1e-6 * delta[d] for d in range(3)]
    delta = [(hi[d] - lo[d]) / (n[d] - 1) for d in range(3)]
    delta = [1e-6 if d == 0 else d for d in delta]  # :145-149
    return OMesh(grid_size, lo, hi, delta, gamma, total_charge, T)


def mesh_manual(grid_size, min_bounds, max_bounds, T=np.float64, gamma=1.0, total_charge=0.0):
    """Manual-bounds constructor, src/mesh.jl:196-238."""
    _check_grid(grid_size)
    if any(float(h) <= float(l) for l, h in zip(min_bounds, max_bounds)):  # :209-211
        raise ValueError("max_bounds must be strictly greater than min_bounds for all dimensions.")
    Tt = np.dtype(T).type
    lo = [Tt(v) for v in min_bounds]
    hi = [Tt(v) for v in max_bounds]
    delta = [(hi[d] - lo[d]) / Tt(int(grid_size[d]) - 1) for d in range(3)]  # :220
    return OMesh(grid_size, lo, hi, delta, gamma, total_charge, T)


def clear_mesh(mesh: OMesh):
    """src/deposition.jl:10-12."""
    mesh.rho[...] = 0


def cic_cells(mesh: OMesh, px, py, pz):
    """Cell index and in-cell fraction, src/deposition.jl:39-51 (and
    src/interpolation.jl:31-43, the same arithmetic).  Returns (i, f) with
    i: int64 (3, Np) 0-based lower-corner node and f: (3, Np) fractions."""
    pts = (np.asarray(px), np.asarray(py), np.asarray(pz))
    idx, frac = [], []
    for d in range(3):
        dt = np.result_type(pts[d].dtype, mesh.T)
        norm = (pts[d].astype(dt) - dt.type(mesh.min_bounds[d])) / dt.type(mesh.delta[d])
        i = np.floor(norm).astype(np.int64)
        idx.append(i)
        frac.append(norm - i)
    return np.stack(idx), np.stack(frac)


def deposit(mesh: OMesh, px, py, pz, pq, clear=True):
    """Serial CIC scatter, src/deposition.jl:218-247 -> :167-197 -> :28-86.

    np.add.at applies the 8 adds per particle in exactly the reference's serial
    order (particle by particle, corners in the order of :77-84), so the FP64
    result is bitwise that of the single-threaded CPU loop.
    """
    px, py, pz, pq = (np.asarray(a) for a in (px, py, pz, pq))
    if not (px.size == py.size == pz.size == pq.size):  # :226-228
        raise ValueError("Particle coordinate and charge arrays must have the same length.")
    if clear:
        clear_mesh(mesh)
    if px.size == 0:
        return
    (ix, iy, iz), (dx, dy, dz) = cic_cells(mesh, px, py, pz)
    nx, ny, nz = mesh.grid_size
    if (ix.min() < 0 or iy.min() < 0 or iz.min() < 0 or ix.max() + 1 >= nx
            or iy.max() + 1 >= ny or iz.max() + 1 >= nz):
        # The reference has no bounds check (deposition.jl:64): out-of-range
        # particles are undefined behaviour there.  The oracle refuses them.
        raise IndexError("particle outside the mesh")
    wx0, wx1, wy0, wy1, wz0, wz1 = 1 - dx, dx, 1 - dy, dy, 1 - dz, dz  # :54-59
    q = pq
    # corners in the order of deposition.jl:67-74, value charge*w_x*w_y*w_z
    corners = [
        (0, 0, 0, q * wx0 * wy0 * wz0), (1, 0, 0, q * wx1 * wy0 * wz0),
        (0, 1, 0, q * wx0 * wy1 * wz0), (1, 1, 0, q * wx1 * wy1 * wz0),
        (0, 0, 1, q * wx0 * wy0 * wz1), (1, 0, 1, q * wx1 * wy0 * wz1),
        (0, 1, 1, q * wx0 * wy1 * wz1), (1, 1, 1, q * wx1 * wy1 * wz1),
    ]
    flat = np.empty((px.size, 8), dtype=np.int64)
    vals = np.empty((px.size, 8), dtype=np.result_type(corners[0][3], np.float64))
    for c, (ox, oy, oz, v) in enumerate(corners):
        flat[:, c] = (ix + ox) + nx * ((iy + oy) + ny * (iz + oz))
        vals[:, c] = v
    r = mesh.rho.reshape(-1, order="F")  # a view: rho is Fortran-contiguous
    if mesh.T == np.float64:
        np.add.at(r, flat.ravel(), vals.ravel())
    else:
        # rho[i] += v with a Float32 rho promotes the add to Float64 and
        # rounds on store (Julia semantics); do the same element-wise.
        acc = r.astype(np.float64)
        np.add.at(acc, flat.ravel(), vals.ravel())
        r[...] = acc.astype(mesh.T)


def field_green_function(x, y, z):
    """Antiderivative of x/r^3, src/green_functions.jl:35-38 (same expression
    and association)."""
    r = np.sqrt(x ** 2 + y ** 2 + z ** 2)
    return x * np.arctan((y * z) / (r * x)) - z * np.log(r + y) + y * np.log((r - z) / (r + z)) / 2


def green_function(shape2, delta, gamma, icomp, offset=(0.0, 0.0, 0.0), T=np.float64):
    """Integrated Green function on the doubled grid for component icomp
    (1, 2, 3), src/green_functions.jl:41-67 with the point kernel :69-101 and
    the 8-point difference :103-112.  Planes isize, jsize, ksize keep the raw
    antiderivative, exactly as the reference leaves them."""
    T = np.dtype(T).type
    isize, jsize, ksize = shape2
    dx, dy, dz = T(delta[0]), T(delta[1]), T(delta[2]) * T(gamma)  # :73
    if icomp in (1, 2):  # :76-80
        factor = T(gamma) / (dx * dy * dz)
    else:
        factor = T(1) / (dx * dy * dz)
    umin = T(1 - isize) * dx / T(2) + T(offset[0])  # :82-84
    vmin = T(1 - jsize) * dy / T(2) + T(offset[1])
    wmin = T(1 - ksize) * dz / T(2) + T(offset[2]) * T(gamma)
    u = (np.arange(isize, dtype=T)) * dx + umin  # :86-88, (i-1) with i 1-based
    v = (np.arange(jsize, dtype=T)) * dy + vmin
    w = (np.arange(ksize, dtype=T)) * dz + wmin
    U, V, W = np.meshgrid(u, v, w, indexing="ij")
    with np.errstate(divide="ignore", invalid="ignore"):
        if icomp == 1:  # :90-98
            g = field_green_function(U, V, W) * factor
        elif icomp == 2:
            g = field_green_function(V, W, U) * factor
        else:
            g = field_green_function(W, U, V) * factor
    g = np.asfortranarray(g.astype(T))
    out = g.copy(order="F")
    out[:-1, :-1, :-1] = (g[1:, 1:, 1:] - g[:-1, 1:, 1:] - g[1:, :-1, 1:] - g[1:, 1:, :-1]
                          - g[:-1, :-1, :-1] + g[:-1, :-1, 1:] + g[:-1, 1:, :-1] + g[1:, :-1, :-1])
    return out


def solve_freespace(mesh: OMesh, offset=(0.0, 0.0, 0.0), rho=None):
    """src/solvers/free_space.jl:56-101: pad -> FFT -> per component
    (IGF, FFT, multiply, IFFT, window extract x FPEI).  Returns efield."""
    nx, ny, nz = mesh.grid_size
    T = mesh.T
    C = np.complex128 if T == np.float64 else np.complex64
    crho = np.zeros((2 * nx, 2 * ny, 2 * nz), dtype=C, order="F")  # :68
    crho[:nx, :ny, :nz] = mesh.rho if rho is None else rho  # :69
    crho = sfft.fftn(crho, workers=_WORKERS)  # :72
    factr = T.type(FPEI)  # :75
    ef = np.zeros(mesh.grid_size + (3,), dtype=T, order="F")
    for icomp in (1, 2, 3):
        g = green_function(crho.shape, mesh.delta, mesh.gamma, icomp, offset, T)
        cgrn = sfft.fftn(g.astype(C), workers=_WORKERS)  # :89
        tmp = crho * cgrn  # :92
        tmp = sfft.ifftn(tmp, workers=_WORKERS)  # :95 (normalised 1/(8N))
        ef[:, :, :, icomp - 1] = factr * np.real(tmp[nx - 1:2 * nx - 1, ny - 1:2 * ny - 1, nz - 1:2 * nz - 1])  # :98-99
    return ef


def solve(mesh: OMesh, at_cathode=False):
    """src/solvers/free_space.jl:14-47, including the image-charge path."""
    T = mesh.T.type
    mesh.efield[...] = solve_freespace(mesh, (T(0), T(0), T(0)))
    if at_cathode:
        image_rho = -mesh.rho[:, :, ::-1]  # :34
        offset_z = T(2) * mesh.min_bounds[2] + (mesh.max_bounds[2] - mesh.min_bounds[2])  # :39
        mesh.efield[...] += solve_freespace(mesh, (T(0), T(0), offset_z), rho=image_rho)  # :42-45


def interpolate_field(mesh: OMesh, px, py, pz):
    """Trilinear gather, src/interpolation.jl:17-86 / :100-128.  Output dtype
    is the particle dtype (similar(particles_x), :110-112)."""
    px = np.asarray(px)
    (ix, iy, iz), (dx, dy, dz) = cic_cells(mesh, px, py, pz)
    nx, ny, nz = mesh.grid_size
    if px.size and (ix.min() < 0 or iy.min() < 0 or iz.min() < 0 or ix.max() + 1 >= nx
                    or iy.max() + 1 >= ny or iz.max() + 1 >= nz):
        raise IndexError("particle outside the mesh")
    w = [
        (0, 0, 0, (1 - dx) * (1 - dy) * (1 - dz)), (1, 0, 0, dx * (1 - dy) * (1 - dz)),
        (0, 1, 0, (1 - dx) * dy * (1 - dz)), (1, 1, 0, dx * dy * (1 - dz)),
        (0, 0, 1, (1 - dx) * (1 - dy) * dz), (1, 0, 1, dx * (1 - dy) * dz),
        (0, 1, 1, (1 - dx) * dy * dz), (1, 1, 1, dx * dy * dz),
    ]  # :46-53
    out = []
    for c in range(3):
        e = mesh.efield[:, :, :, c]
        acc = None
        for ox, oy, oz, wt in w:  # :56-85, left-to-right sum
            term = e[ix + ox, iy + oy, iz + oz] * wt
            acc = term if acc is None else acc + term
        if acc is None:
            acc = np.zeros(0)
        out.append(np.asarray(acc).astype(px.dtype))
    return tuple(out)


def kick(mesh: OMesh, px, py, pz, pq, at_cathode=False):
    """deposit! -> solve! -> interpolate_field, the unit timed by
    benchmark/full_pipeline_benchmark.jl:26-30."""
    deposit(mesh, px, py, pz, pq)
    solve(mesh, at_cathode=at_cathode)
    return interpolate_field(mesh, px, py, pz)


def linear_green_kernel(mesh: OMesh, icomp, offset=(0.0, 0.0, 0.0)):
    """The part of green_function() that the output window reads, indexed by
    the displacement d in [-(n-1), n-1] per axis: returns K of shape
    (2nx-1, 2ny-1, 2nz-1) with K[d + n - 1] = G[d + n - 1] (0-based cell
    index c = d + n - 1, see free_space.jl:98-99)."""
    nx, ny, nz = mesh.grid_size
    g = green_function((2 * nx, 2 * ny, 2 * nz), mesh.delta, mesh.gamma, icomp, offset, mesh.T)
    return g[:-1, :-1, :-1]


def gaussian_field(x, y, z, Q, sigma):
    """Exact field of an isotropic Gaussian bunch, test/analytical_test.jl:12-17."""
    r = np.sqrt(x * x + y * y + z * z)
    with np.errstate(divide="ignore", invalid="ignore"):
        erf = np.vectorize(math.erf)(r / (math.sqrt(2) * sigma)) if np.ndim(r) else math.erf(r / (math.sqrt(2) * sigma))
        s = Q / (4 * math.pi * EPSILON_0 * r ** 3) * (erf - math.sqrt(2 / math.pi) * r / sigma * np.exp(-(r / sigma) ** 2 / 2))
        s = np.where(r == 0, 0.0, s)
    return s * x, s * y, s * z


# ------------------------------------------------ beside the kick (no reference code)
# The rows next to the kick: the bunch's magnetic field and the tracking step
# that calls the kick.  The reference package has neither; these restate the
# library's documented definitions so its GPU path has an FP64 checker.
def magnetic_field(mesh: OMesh, ex, ey):
    """B of a bunch moving along +z at the mesh's gamma: B = (beta/c) z x E,
    Bx = -beta Ey / c, By = beta Ex / c, Bz = 0."""
    beta = math.sqrt(1.0 - 1.0 / (mesh.gamma * mesh.gamma))
    k = beta / CLIGHT
    return -k * np.asarray(ey, np.float64), k * np.asarray(ex, np.float64)


def boris_push(x, y, z, ux, uy, uz, ex, ey, ez, bx, by, dt, qm):
    """One relativistic Boris step (J. P. Boris 1970; Birdsall & Langdon,
    Plasma Physics via Computer Simulation, section 15-4) of u = gamma*beta
    (dimensionless) under SI fields E [V/m], B = (bx, by, 0) [T], for a
    species of charge/mass qm [C/kg], then the drift x += c u/gamma dt.
    du/dt = qm/c (E + v x B); all arrays FP64, returns the new state."""
    a = qm * dt / (2.0 * CLIGHT)  # half electric kick, in units of u per V/m
    umx, umy, umz = ux + a * ex, uy + a * ey, uz + a * ez
    g = np.sqrt(1.0 + umx * umx + umy * umy + umz * umz)
    tb = qm * dt / (2.0 * g)
    tx, ty = tb * bx, tb * by  # tz = 0
    # u' = u- + u- x t
    upx = umx - umz * ty
    upy = umy + umz * tx
    upz = umz + (umx * ty - umy * tx)
    s = 2.0 / (1.0 + tx * tx + ty * ty)
    sx, sy = s * tx, s * ty
    # u+ = u- + u' x s
    upl_x = umx - upz * sy
    upl_y = umy + upz * sx
    upl_z = umz + (upx * sy - upy * sx)
    nx, ny, nz = upl_x + a * ex, upl_y + a * ey, upl_z + a * ez
    gn = np.sqrt(1.0 + nx * nx + ny * ny + nz * nz)
    f = CLIGHT * dt / gn
    return x + f * nx, y + f * ny, z + f * nz, nx, ny, nz


def track(grid_size, x, y, z, ux, uy, uz, q, dt, qm, steps, gamma=1.0, at_cathode=False):
    """`steps` tracking steps of a bunch in its own field: refit a mesh to
    the particles (the particle constructor, mesh.jl:95-174), kick, B from
    E, one Boris step.  Returns the final (x, y, z, ux, uy, uz)."""
    state = [np.array(a, dtype=np.float64) for a in (x, y, z, ux, uy, uz)]
    for _ in range(steps):
        m = mesh_auto(grid_size, state[0], state[1], state[2], gamma=gamma)
        ex, ey, ez = kick(m, state[0], state[1], state[2], q, at_cathode=at_cathode)
        bx, by = magnetic_field(m, ex, ey)
        state = list(boris_push(*state, ex, ey, ez, bx, by, dt, qm))
    return tuple(state)


# ------------------------------------------------ scalar potential (reference code unused)
def potential_green_function(x, y, z):
    """Antiderivative of 1/r, src/green_functions.jl:13-22 (defined in the
    reference, never called): zero at r = 0, same expression and order."""
    r = np.sqrt(x ** 2 + y ** 2 + z ** 2)
    half = 0.5
    with np.errstate(divide="ignore", invalid="ignore"):
        v = (-half * z ** 2 * np.arctan(x * y / (z * r)) - half * y ** 2 * np.arctan(x * z / (y * r))
             - half * x ** 2 * np.arctan(y * z / (x * r)) + y * z * np.log(x + r)
             + x * z * np.log(y + r) + x * y * np.log(z + r))
    return np.where(r == 0, 0.0, v)


def potential_green(shape2, delta, gamma, offset=(0.0, 0.0, 0.0)):
    """Integrated potential Green function on the doubled grid: the corner
    lattice, gamma scaling and 8-point difference of green_function() with
    potential_green_function and the transverse factor gamma/(dx dy dz), so
    that the solve gives the lab-frame potential gamma*phi' of the bunch's
    rest-frame potential phi' (the time component of the four-potential)."""
    isize, jsize, ksize = shape2
    dx, dy, dz = float(delta[0]), float(delta[1]), float(delta[2]) * float(gamma)
    factor = float(gamma) / (dx * dy * dz)
    umin = (1 - isize) * dx / 2 + float(offset[0])
    vmin = (1 - jsize) * dy / 2 + float(offset[1])
    wmin = (1 - ksize) * dz / 2 + float(offset[2]) * float(gamma)
    u = np.arange(isize) * dx + umin
    v = np.arange(jsize) * dy + vmin
    w = np.arange(ksize) * dz + wmin
    U, V, W = np.meshgrid(u, v, w, indexing="ij")
    g = np.asfortranarray(potential_green_function(U, V, W) * factor)
    out = g.copy(order="F")
    out[:-1, :-1, :-1] = (g[1:, 1:, 1:] - g[:-1, 1:, 1:] - g[1:, :-1, 1:] - g[1:, 1:, :-1]
                          - g[:-1, :-1, :-1] + g[:-1, :-1, 1:] + g[:-1, 1:, :-1] + g[1:, :-1, :-1])
    return out


def _solve_potential_freespace(mesh: OMesh, offset, rho):
    nx, ny, nz = mesh.grid_size
    crho = np.zeros((2 * nx, 2 * ny, 2 * nz), dtype=np.complex128, order="F")
    crho[:nx, :ny, :nz] = rho
    crho = sfft.fftn(crho, workers=_WORKERS)
    cgrn = sfft.fftn(potential_green(crho.shape, mesh.delta, mesh.gamma, offset).astype(np.complex128),
                     workers=_WORKERS)
    tmp = sfft.ifftn(crho * cgrn, workers=_WORKERS)
    return FPEI * np.real(tmp[nx - 1:2 * nx - 1, ny - 1:2 * ny - 1, nz - 1:2 * nz - 1])


def solve_potential(mesh: OMesh, at_cathode=False):
    """Scalar potential on the mesh from mesh.rho, the schedule of solve()
    (free_space.jl:14-101) with the potential Green function; the cathode
    image enters as in the field solve (-rho flipped in z, offset zmin+zmax)."""
    phi = _solve_potential_freespace(mesh, (0.0, 0.0, 0.0), mesh.rho)
    if at_cathode:
        offset_z = 2.0 * mesh.min_bounds[2] + (mesh.max_bounds[2] - mesh.min_bounds[2])
        phi = phi + _solve_potential_freespace(mesh, (0.0, 0.0, offset_z), -mesh.rho[:, :, ::-1])
    return phi


def gaussian_potential(x, y, z, Q, sigma):
    """Exact potential of an isotropic Gaussian bunch: Q/(4 pi eps0 r) erf(r/(sqrt2 sigma)),
    Q sqrt(2/pi)/(4 pi eps0 sigma) at r = 0."""
    r = np.sqrt(np.asarray(x) ** 2 + np.asarray(y) ** 2 + np.asarray(z) ** 2)
    k = Q / (4 * math.pi * EPSILON_0)
    with np.errstate(divide="ignore", invalid="ignore"):
        erf = np.vectorize(math.erf)(r / (math.sqrt(2) * sigma))
        v = k * erf / r
    return np.where(r == 0, k * math.sqrt(2 / math.pi) / sigma, v)
