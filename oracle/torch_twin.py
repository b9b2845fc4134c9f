"""Differentiable FP64 torch twin of the oracle's kick (test infrastructure).

The same arithmetic as sc_oracle.kick -- CIC deposit (src/deposition.jl:28-86),
the reference's doubled-grid c2c FFT solve with its integrated Green function
(src/solvers/free_space.jl:14-101, src/green_functions.jl:41-112) and the
trilinear gather (src/interpolation.jl:17-86) -- written with torch ops so
that autograd gives d(loss)/d(x, y, z, q) with the mesh geometry fixed.  The
reference itself cannot be differentiated by ForwardDiff (its Mesh3D element
type is restricted to AbstractFloat, src/mesh.jl:100); this twin stands in
for that check.  Used only by tests.
"""
from __future__ import annotations

import numpy as np
import torch

from . import sc_oracle as O


def _cells(p, lo, delta):
    norm = (p - lo) / delta
    i = torch.floor(norm.detach())
    return i.long(), norm - i


def _corners(nx, ny):
    return [(a, b, c) for c in (0, 1) for b in (0, 1) for a in (0, 1)]


def kick(mesh: O.OMesh, x, y, z, q, at_cathode=False):
    """Returns (Ex, Ey, Ez) at the particles and the mesh efield (nx,ny,nz,3),
    differentiable with respect to x, y, z, q (torch float64 tensors)."""
    nx, ny, nz = mesh.grid_size
    lo, dl = mesh.min_bounds, mesh.delta
    (ix, fx), (iy, fy), (iz, fz) = (_cells(p, float(lo[d]), float(dl[d])) for d, p in enumerate((x, y, z)))
    wx = (1 - fx, fx)
    wy = (1 - fy, fy)
    wz = (1 - fz, fz)
    rho = torch.zeros(nx * ny * nz, dtype=torch.float64)
    for a, b, c in _corners(nx, ny):
        idx = (ix + a) + nx * ((iy + b) + ny * (iz + c))
        rho = rho.index_add(0, idx, q * wx[a] * wy[b] * wz[c])
    rho3 = rho.reshape(nz, ny, nx).permute(2, 1, 0)  # (nx, ny, nz)

    def solve_free(r, offset):
        crho = torch.zeros((2 * nx, 2 * ny, 2 * nz), dtype=torch.complex128)
        crho[:nx, :ny, :nz] = r.to(torch.complex128)
        R = torch.fft.fftn(crho)
        out = []
        for icomp in (1, 2, 3):
            g = O.green_function((2 * nx, 2 * ny, 2 * nz), mesh.delta, mesh.gamma, icomp, offset)
            G = torch.fft.fftn(torch.from_numpy(np.ascontiguousarray(g)).to(torch.complex128))
            e = torch.fft.ifftn(R * G).real[nx - 1:2 * nx - 1, ny - 1:2 * ny - 1, nz - 1:2 * nz - 1]
            out.append(O.FPEI * e)
        return torch.stack(out, dim=-1)

    E = solve_free(rho3, (0.0, 0.0, 0.0))
    if at_cathode:
        offz = 2 * float(lo[2]) + (float(mesh.max_bounds[2]) - float(lo[2]))
        E = E + solve_free(-torch.flip(rho3, dims=(2,)), (0.0, 0.0, offz))
    Ef = E.permute(2, 1, 0, 3).reshape(-1, 3)
    outs = []
    for comp in range(3):
        acc = 0
        for a, b, c in _corners(nx, ny):
            idx = (ix + a) + nx * ((iy + b) + ny * (iz + c))
            acc = acc + Ef[idx, comp] * (wx[a] * wy[b] * wz[c])
        outs.append(acc)
    return outs[0], outs[1], outs[2], E
