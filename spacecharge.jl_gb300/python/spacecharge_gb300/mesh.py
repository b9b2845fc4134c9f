"""Python host of the GB300 space-charge kick, mirroring SpaceCharge.jl's
public API (src/SpaceCharge.jl:17): Mesh3D, deposit (deposit!), clear_mesh
(clear_mesh!), solve (solve!) and interpolate_field, with the same argument
meaning and error behaviour.  All compute runs in libspacecharge_gb300.so;
torch supplies device memory and the current CUDA stream."""
from __future__ import annotations

import ctypes as C
from typing import Sequence

import numpy as np

from . import _lib as L
from ._lib import SpaceChargeError

CLIGHT = 299792458.0  # src/utils.jl:7
FPEI = CLIGHT ** 2 * 1.0e-7  # src/utils.jl:8

_PRECISIONS = {"plain64": L.SC_PREC_PLAIN64, "fp64": L.SC_PREC_FP64, "mixed": L.SC_PREC_MIXED}
_MODES = {"atomic": L.SC_DEPOSIT_ATOMIC, "sorted": L.SC_DEPOSIT_SORTED,
          "deterministic": L.SC_DEPOSIT_DETERMINISTIC, "tiled": L.SC_DEPOSIT_TILED,
          "vector": L.SC_DEPOSIT_VECTOR}


def _torch():
    import torch
    return torch


def _stream():
    torch = _torch()
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def _length(a) -> int:
    return int(a.numel()) if hasattr(a, "numel") else int(np.asarray(a).size)


def _is_device_tensor(a) -> bool:
    return hasattr(a, "is_cuda") and bool(a.is_cuda)


def _as_device(arrays, dtype=None):
    """Particle arrays -> contiguous CUDA tensors of one float dtype (the
    promoted type, as Julia promotes mixed element types)."""
    torch = _torch()
    ts = []
    for a in arrays:
        if isinstance(a, torch.Tensor):
            t = a
        else:
            t = torch.from_numpy(np.ascontiguousarray(np.asarray(a)))
        ts.append(t)
    if dtype is None:
        dtype = torch.float64 if any(t.dtype == torch.float64 for t in ts) else torch.float32
        if any(not t.is_floating_point() for t in ts):
            dtype = torch.float64
    out = []
    for t in ts:
        if t.dtype != dtype:
            t = t.to(dtype)
        if not t.is_cuda:
            t = t.pin_memory().cuda(non_blocking=True) if t.numel() else t.cuda()
        out.append(t.contiguous())
    return out, (L.SC_F64 if dtype == torch.float64 else L.SC_F32)


class _CudaView:
    """__cuda_array_interface__ over mesh-owned memory; keeps the mesh alive."""

    def __init__(self, handle, ptr, shape, typestr):
        self._handle = handle
        self.__cuda_array_interface__ = {"shape": tuple(shape), "typestr": typestr, "data": (ptr, False),
                                         "version": 2, "strides": None}


class _Handle:
    def __init__(self, ptr: C.c_void_p):
        self.ptr = ptr

    def __del__(self):
        if self.ptr and self.ptr.value and L._lib is not None:
            L._lib.sc_mesh_destroy(self.ptr)
            self.ptr = None


class Mesh3D:
    """Mesh3D(grid_size, particles_x, particles_y, particles_z; ...) or
    Mesh3D(grid_size, min_bounds, max_bounds; ...), src/mesh.jl:95-238.

    Keywords: T (np.float64 -> precision "fp64", np.float32 -> "mixed"),
    precision ("plain64" = the reference algorithm in FP64 with cuFFT,
    "fp64", "mixed"), gamma, total_charge.
    """

    def __init__(self, grid_size: Sequence[int], *args, T=np.float64, precision: str | None = None,
                 gamma: float = 1.0, total_charge: float = 0.0):
        if len(grid_size) != 3:
            raise SpaceChargeError("grid_size must have 3 elements")
        if precision is None:
            precision = "fp64" if np.dtype(T) == np.float64 else "mixed"
        if precision not in _PRECISIONS:
            raise SpaceChargeError(f"unknown precision {precision!r}")
        self.precision = precision
        g = (C.c_int32 * 3)(*[int(v) for v in grid_size])
        out = C.c_void_p()
        prec = _PRECISIONS[precision]
        if len(args) == 2:  # manual bounds, mesh.jl:196-238
            lo = (C.c_double * 3)(*[float(v) for v in args[0]])
            hi = (C.c_double * 3)(*[float(v) for v in args[1]])
            L.call("sc_mesh_create", g, lo, hi, float(gamma), float(total_charge), prec, C.byref(out))
        elif len(args) == 3:  # particle bounds, mesh.jl:95-174
            if any(int(v) <= 1 for v in grid_size):  # :106-108
                raise SpaceChargeError("All elements of grid_size must be at least 2.")
            lens = [_length(a) for a in args]
            if min(lens) == 0:  # :110-112
                raise SpaceChargeError("Particle arrays cannot be empty.")
            if not (lens[0] == lens[1] == lens[2]):  # :114-116
                raise SpaceChargeError("Particle coordinate arrays must have the same length.")
            (x, y, z), dt = _as_device(args)
            L.call("sc_mesh_create_from_particles", g, C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()),
                   C.c_void_p(z.data_ptr()), lens[0], dt, float(gamma), float(total_charge), prec, _stream(),
                   C.byref(out))
        else:
            raise SpaceChargeError("Mesh3D(grid_size, px, py, pz) or Mesh3D(grid_size, min_bounds, max_bounds)")
        self._h = _Handle(out)
        self._refresh()
        self._rho = None
        self._efield = None

    def _refresh(self) -> None:
        """Re-read the mesh's properties (after a change of bounds)."""
        info = L.MeshInfo()
        L.call("sc_mesh_get_info", self._h.ptr, C.byref(info))
        self.grid_size = tuple(int(v) for v in info.grid_size)
        self.min_bounds = tuple(float(v) for v in info.min_bounds)
        self.max_bounds = tuple(float(v) for v in info.max_bounds)
        self.delta = tuple(float(v) for v in info.delta)
        self.gamma = float(info.gamma)
        self.total_charge = float(info.total_charge)
        self.fft_shape = tuple(int(v) for v in info.fft_shape)
        self.efield_layout = int(info.efield_layout)
        self.T = np.float32 if info.elem_bytes == 4 else np.float64

    def set_bounds(self, min_bounds, max_bounds) -> None:
        """New bounds for this mesh, keeping its grid, fields and workspaces
        (sc_mesh_set_bounds; the manual constructor's validation and delta)."""
        lo = (C.c_double * 3)(*[float(v) for v in min_bounds])
        hi = (C.c_double * 3)(*[float(v) for v in max_bounds])
        L.call("sc_mesh_set_bounds", self._h.ptr, lo, hi)
        self._refresh()

    def refit(self, particles_x, particles_y, particles_z) -> None:
        """The particle constructor's bounds for these particles
        (sc_mesh_refit, src/mesh.jl:95-174)."""
        lens = [_length(a) for a in (particles_x, particles_y, particles_z)]
        if min(lens) == 0:
            raise SpaceChargeError("Particle arrays cannot be empty.")
        if not (lens[0] == lens[1] == lens[2]):
            raise SpaceChargeError("Particle coordinate arrays must have the same length.")
        (x, y, z), dt = _as_device((particles_x, particles_y, particles_z))
        L.call("sc_mesh_refit", self._h.ptr, C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()),
               C.c_void_p(z.data_ptr()), lens[0], dt, _stream())
        self._refresh()

    # --- field access (mesh.rho / mesh.efield in the reference) -----------
    @property
    def ptr(self):
        return self._h.ptr

    @property
    def rho(self):
        """Device view of rho with shape (nx, ny, nz) (x fastest, as Julia)."""
        if self._rho is None:
            torch = _torch()
            p = C.c_void_p()
            L.call("sc_mesh_rho", self._h.ptr, C.byref(p))
            nx, ny, nz = self.grid_size
            ts = "<f4" if self.T == np.float32 else "<f8"
            base = torch.as_tensor(_CudaView(self._h, p.value, (nz, ny, nx), ts), device="cuda")
            self._rho = base.permute(2, 1, 0)
        return self._rho

    @property
    def efield(self):
        """Device view of efield with shape (nx, ny, nz, 3)."""
        if self._efield is None:
            torch = _torch()
            p = C.c_void_p()
            L.call("sc_mesh_efield", self._h.ptr, C.byref(p))
            nx, ny, nz = self.grid_size
            ts = "<f4" if self.T == np.float32 else "<f8"
            if self.efield_layout == L.SC_LAYOUT_PACKED:
                base = torch.as_tensor(_CudaView(self._h, p.value, (nz, ny, nx, 4), ts), device="cuda")
                self._efield = base.permute(2, 1, 0, 3)[..., :3]
            else:
                base = torch.as_tensor(_CudaView(self._h, p.value, (3, nz, ny, nx), ts), device="cuda")
                self._efield = base.permute(3, 2, 1, 0)
        return self._efield

    def set_kick_mode(self, mode: str) -> None:
        """Deposit mode used by kick(): "vector" (default for mixed meshes),
        "atomic" (default otherwise), "tiled" (the kick then also gathers
        through the same tiles), "sorted" or "deterministic"."""
        if mode not in _MODES:
            raise SpaceChargeError(f"unknown deposit mode {mode!r}")
        L.call("sc_mesh_set_kick_mode", self._h.ptr, _MODES[mode])

    def launch_count(self) -> int:
        """Kernels this mesh's calls have launched (graph replays included)."""
        n = C.c_int64()
        L.call("sc_mesh_launch_count", self._h.ptr, C.byref(n))
        return int(n.value)

    def set_kick_graph(self, enabled: bool) -> None:
        """Replay repeated kick() calls with the same particle and output
        arrays as one CUDA graph launch (default on)."""
        L.call("sc_mesh_set_kick_graph", self._h.ptr, 1 if enabled else 0)

    def set_green_cache(self, enabled: bool) -> None:
        L.call("sc_mesh_set_green_cache", self._h.ptr, 1 if enabled else 0)

    def set_fp64_arithmetic(self, mode: str) -> None:
        """precision="fp64" meshes: "fp64" (default) runs the kick in FP64;
        "df32" runs the atomic deposit's weights, the x, y and (free-space) z
        transform passes and the interpolation in double-FP32 (48-bit
        significands, about 1e-14 of the fields' maximum)."""
        modes = {"fp64": L.SC_FP64_ARITH_FP64, "df32": L.SC_FP64_ARITH_DF32}
        if mode not in modes:
            raise ValueError(f"unknown FP64 transform mode {mode!r}")
        L.call("sc_mesh_set_fp64_arithmetic", self._h.ptr, modes[mode])

    def out_of_range(self) -> int:
        """Particles skipped as outside the mesh since the last query."""
        n = C.c_int64()
        L.call("sc_mesh_out_of_range", self._h.ptr, C.byref(n), _stream())
        return int(n.value)

    def __repr__(self):  # mesh.jl:240-246
        nx, ny, nz = self.grid_size
        lo, hi = self.min_bounds, self.max_bounds
        T = "Float32" if self.T == np.float32 else "Float64"
        return (f"Mesh3D{{{T}, {self.precision}}} ({nx}x{ny}x{nz}) bounds=[({lo[0]},{lo[1]},{lo[2]}), "
                f"({hi[0]},{hi[1]},{hi[2]})] gamma={self.gamma}")


def clear_mesh(mesh: Mesh3D) -> None:
    """clear_mesh!(mesh), src/deposition.jl:10-12."""
    L.call("sc_clear_mesh", mesh.ptr, _stream())


def deposit(mesh: Mesh3D, particles_x, particles_y, particles_z, particles_q, clear: bool = True,
            mode: str = "atomic") -> None:
    """deposit!(mesh, px, py, pz, pq; clear=true), src/deposition.jl:218-247."""
    lens = [_length(a) for a in (particles_x, particles_y, particles_z, particles_q)]
    if not (lens[0] == lens[1] == lens[2] == lens[3]):  # :226-228
        raise SpaceChargeError("Particle coordinate and charge arrays must have the same length.")
    if mode not in _MODES:
        raise SpaceChargeError(f"unknown deposit mode {mode!r}")
    if lens[0] == 0:
        if clear:
            clear_mesh(mesh)
        return
    (x, y, z, q), dt = _as_device((particles_x, particles_y, particles_z, particles_q))
    L.call("sc_deposit", mesh.ptr, C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()), C.c_void_p(z.data_ptr()),
           C.c_void_p(q.data_ptr()), lens[0], dt, 1 if clear else 0, _MODES[mode], _stream())


def solve(mesh: Mesh3D, at_cathode: bool = False) -> None:
    """solve!(mesh; at_cathode=false), src/solvers/free_space.jl:14-47."""
    L.call("sc_solve", mesh.ptr, 1 if at_cathode else 0, _stream())


def _similar_out(template, xs):
    """Outputs of the particle type and array kind (similar(particles_x))."""
    torch = _torch()
    return [torch.empty_like(xs[0]) for _ in range(3)]


def _return_like(template, outs):
    torch = _torch()
    if isinstance(template, torch.Tensor):
        return tuple(o if template.is_cuda else o.cpu() for o in outs)
    return tuple(o.cpu().numpy() for o in outs)


def interpolate_field(mesh: Mesh3D, particles_x, particles_y, particles_z):
    """interpolate_field(mesh, px, py, pz) -> (Ex, Ey, Ez),
    src/interpolation.jl:100-128: outputs have the particle element type and
    array kind (device tensors stay on the device, host arrays come back to
    the host)."""
    lens = [_length(a) for a in (particles_x, particles_y, particles_z)]
    if not (lens[0] == lens[1] == lens[2]):
        raise SpaceChargeError("Particle coordinate arrays must have the same length.")
    (x, y, z), dt = _as_device((particles_x, particles_y, particles_z))
    ex, ey, ez = _similar_out(particles_x, (x, y, z))
    if lens[0]:
        L.call("sc_interpolate_field", mesh.ptr, C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()),
               C.c_void_p(z.data_ptr()), lens[0], dt, C.c_void_p(ex.data_ptr()), C.c_void_p(ey.data_ptr()),
               C.c_void_p(ez.data_ptr()), _stream())
    return _return_like(particles_x, (ex, ey, ez))


def kick(mesh: Mesh3D, particles_x, particles_y, particles_z, particles_q, at_cathode: bool = False, out=None):
    """deposit! -> solve! -> interpolate_field in one library call.  `out`:
    three contiguous CUDA tensors of the particle dtype to write the field
    into (repeated calls with the same particle tensors and `out` replay a
    captured CUDA graph)."""
    lens = [_length(a) for a in (particles_x, particles_y, particles_z, particles_q)]
    if not (lens[0] == lens[1] == lens[2] == lens[3]):
        raise SpaceChargeError("Particle coordinate and charge arrays must have the same length.")
    (x, y, z, q), dt = _as_device((particles_x, particles_y, particles_z, particles_q))
    if out is not None:
        ex, ey, ez = out
        for t in out:
            if not (_is_device_tensor(t) and t.is_contiguous() and t.dtype == x.dtype and t.numel() == lens[0]):
                raise SpaceChargeError("out must be three contiguous CUDA tensors of the particle dtype and count")
    else:
        ex, ey, ez = _similar_out(particles_x, (x, y, z))
    L.call("sc_kick", mesh.ptr, C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()), C.c_void_p(z.data_ptr()),
           C.c_void_p(q.data_ptr()), lens[0], dt, 1 if at_cathode else 0, C.c_void_p(ex.data_ptr()),
           C.c_void_p(ey.data_ptr()), C.c_void_p(ez.data_ptr()), _stream())
    if out is not None:
        return tuple(out)
    return _return_like(particles_x, (ex, ey, ez))


def kick_host(mesh: Mesh3D, particles_x, particles_y, particles_z, particles_q, at_cathode: bool = False,
              out=None):
    """kick() for particles in host memory (numpy arrays or CPU tensors):
    the library streams them to the GPU in chunks, overlapping the copies
    with the deposit and the gather (sc_kick_host).  Returns host arrays of
    the particle type (page-locked torch tensors, or `out` if given); the
    call returns when they hold the field."""
    torch = _torch()
    lens = [_length(a) for a in (particles_x, particles_y, particles_z, particles_q)]
    if not (lens[0] == lens[1] == lens[2] == lens[3]):
        raise SpaceChargeError("Particle coordinate and charge arrays must have the same length.")
    ts = [a if isinstance(a, torch.Tensor) else torch.from_numpy(np.ascontiguousarray(np.asarray(a)))
          for a in (particles_x, particles_y, particles_z, particles_q)]
    if any(t.is_cuda for t in ts):
        raise SpaceChargeError("kick_host takes host arrays; use kick() for device arrays")
    dt = torch.float64 if any(t.dtype == torch.float64 for t in ts) else torch.float32
    ts = [t.to(dt).contiguous() for t in ts]
    if out is None:
        out = [torch.empty(lens[0], dtype=dt, pin_memory=True) for _ in range(3)]
    L.call("sc_kick_host", mesh.ptr, *[C.c_void_p(t.data_ptr()) for t in ts], lens[0],
           L.SC_F64 if dt == torch.float64 else L.SC_F32, 1 if at_cathode else 0,
           *[C.c_void_p(o.data_ptr()) for o in out], _stream())
    torch.cuda.current_stream().synchronize()
    return tuple(out)


def solve_potential(mesh: Mesh3D, at_cathode: bool = False):
    """Scalar potential on the mesh nodes from mesh.rho (sc_solve_potential):
    a device tensor of shape (nx, ny, nz) of the mesh type."""
    torch = _torch()
    nx, ny, nz = mesh.grid_size
    dt = torch.float32 if mesh.T == np.float32 else torch.float64
    phi = torch.empty((nz, ny, nx), dtype=dt, device="cuda")
    L.call("sc_solve_potential", mesh.ptr, 1 if at_cathode else 0, _ptr(phi), _stream())
    return phi.permute(2, 1, 0)


def track(mesh: Mesh3D, x, y, z, ux, uy, uz, q, dt: float, qm: float, steps: int = 1, refit: bool = True,
          at_cathode: bool = False) -> None:
    """`steps` tracking steps of the bunch in its own field (sc_track): refit
    the mesh bounds (when `refit`), kick, B from E, one relativistic Boris
    step of u = gamma*beta and the positions over dt [s] for charge/mass qm
    [C/kg].  x, y, z, ux, uy, uz are CUDA tensors of one float type, updated
    in place; q the macro charges."""
    torch = _torch()
    ts = (x, y, z, ux, uy, uz, q)
    if not all(isinstance(t, torch.Tensor) and t.is_cuda and t.is_contiguous() for t in ts):
        raise SpaceChargeError("track updates contiguous CUDA tensors in place")
    if len({t.dtype for t in ts}) != 1 or x.dtype not in (torch.float32, torch.float64):
        raise SpaceChargeError("track needs all arrays float32 or all float64")
    if len({t.numel() for t in ts}) != 1:
        raise SpaceChargeError("Particle coordinate and charge arrays must have the same length.")
    L.call("sc_track", mesh.ptr, *[_ptr(t) for t in ts], x.numel(), L.SC_F64 if x.dtype == torch.float64 else L.SC_F32,
           float(dt), float(qm), int(steps), 1 if refit else 0, 1 if at_cathode else 0, _stream())
    if refit:
        mesh._refresh()


def magnetic_field(mesh: Mesh3D, ex, ey):
    """B at the particles of a bunch moving along +z at the mesh's gamma:
    Bx = -beta Ey / c, By = beta Ex / c, Bz = 0 (sc_magnetic_field).  ex, ey
    are the kick's outputs (device tensors or host arrays)."""
    torch = _torch()
    (tx, ty), dt = _as_device((ex, ey))
    bx, by = torch.empty_like(tx), torch.empty_like(tx)
    L.call("sc_magnetic_field", mesh.ptr, _ptr(tx), _ptr(ty), tx.numel(), dt, _ptr(bx), _ptr(by), _stream())
    return _return_like(ex, (bx, by))


def aos_to_soa(records, offsets=(0, 1, 2, 3)):
    """Particle records (n, stride) on the device -> x, y, z, q arrays
    (sc_aos_to_soa); `offsets` are the record positions of x, y, z, q."""
    torch = _torch()
    r = torch.as_tensor(records, device="cuda").contiguous()
    if r.dim() != 2 or r.dtype not in (torch.float32, torch.float64):
        raise SpaceChargeError("records must be a float32/float64 (n, stride) array")
    n, stride = r.shape
    outs = [torch.empty(n, dtype=r.dtype, device="cuda") for _ in range(4)]
    offs = (C.c_int32 * 4)(*offsets)
    L.call("sc_aos_to_soa", _ptr(r), n, stride, offs, L.SC_F64 if r.dtype == torch.float64 else L.SC_F32,
           *[_ptr(o) for o in outs], _stream())
    return tuple(outs)


def soa_to_aos(ex, ey, ez, records, offsets=(4, 5, 6)):
    """Write the field components into device particle records (n, stride)
    at `offsets` (sc_soa_to_aos)."""
    torch = _torch()
    (tx, ty, tz), dt = _as_device((ex, ey, ez), dtype=records.dtype)
    if not (records.is_cuda and records.is_contiguous() and records.dim() == 2):
        raise SpaceChargeError("records must be a contiguous (n, stride) device tensor")
    offs = (C.c_int32 * 3)(*offsets)
    L.call("sc_soa_to_aos", _ptr(tx), _ptr(ty), _ptr(tz), tx.numel(), dt, records.shape[1], offs, _ptr(records),
           _stream())
    return records


def relative_to_absolute(rx, ry, rz, ref):
    """FP32 positions relative to the FP64 point `ref` -> FP64 absolute
    positions on the device (sc_relative_to_absolute)."""
    torch = _torch()
    (tx, ty, tz), _ = _as_device((rx, ry, rz), dtype=torch.float32)
    outs = [torch.empty(tx.numel(), dtype=torch.float64, device="cuda") for _ in range(3)]
    r = (C.c_double * 3)(*ref)
    L.call("sc_relative_to_absolute", _ptr(tx), _ptr(ty), _ptr(tz), tx.numel(), r, *[_ptr(o) for o in outs],
           _stream())
    return tuple(outs)


def _ptr(t):
    return C.c_void_p(t.data_ptr()) if t is not None else None


def _packed_grid_grad(mesh: Mesh3D, g):
    """dL/d(mesh.efield) given as (nx, ny, nz, 3) -> the mesh's packed
    (nz, ny, nx, 4) device layout of its element type."""
    torch = _torch()
    if mesh.efield_layout != L.SC_LAYOUT_PACKED:
        raise SpaceChargeError("grid gradients need a packed-layout mesh", L.SC_ERR_UNSUPPORTED)
    dt = torch.float32 if mesh.T == np.float32 else torch.float64
    nx, ny, nz = mesh.grid_size
    g = torch.as_tensor(g, dtype=dt, device="cuda")
    if tuple(g.shape) != (nx, ny, nz, 3):
        raise SpaceChargeError(f"grid gradient must have shape {(nx, ny, nz, 3)}")
    out = torch.zeros((nz, ny, nx, 4), dtype=dt, device="cuda")
    out[..., :3] = g.permute(2, 1, 0, 3)
    return out


def kick_adjoint(mesh: Mesh3D, particles_x, particles_y, particles_z, particles_q, gEx=None, gEy=None, gEz=None,
                 gEgrid=None, at_cathode: bool = False):
    """Hand-written adjoint of kick(): d(loss)/d(x, y, z, q) from the
    upstream gradients d(loss)/d(Ex, Ey, Ez) at the particles and, optionally,
    d(loss)/d(mesh.efield) of shape (nx, ny, nz, 3).  Recomputes the forward
    deposit and solve.  Returns device tensors of the particle dtype."""
    torch = _torch()
    lens = [_length(a) for a in (particles_x, particles_y, particles_z, particles_q)]
    if not (lens[0] == lens[1] == lens[2] == lens[3]):
        raise SpaceChargeError("Particle coordinate and charge arrays must have the same length.")
    (x, y, z, q), dt = _as_device((particles_x, particles_y, particles_z, particles_q))
    tdt = x.dtype
    gs = []
    for g in (gEx, gEy, gEz):
        if g is None:
            gs.append(None)
        else:
            t, _ = _as_device((g,), dtype=tdt)
            if t[0].numel() != lens[0]:
                raise SpaceChargeError("field gradients must have one entry per particle")
            gs.append(t[0])
    gg = _packed_grid_grad(mesh, gEgrid) if gEgrid is not None else None
    outs = [torch.empty_like(x) for _ in range(4)]
    L.call("sc_kick_adjoint", mesh.ptr, _ptr(x), _ptr(y), _ptr(z), _ptr(q), lens[0], dt, 1 if at_cathode else 0,
           _ptr(gs[0]), _ptr(gs[1]), _ptr(gs[2]), _ptr(gg), *[_ptr(o) for o in outs], _stream())
    return tuple(outs)


def _make_kick_function():
    torch = _torch()

    class KickFunction(torch.autograd.Function):
        """(x, y, z, q) -> (Ex, Ey, Ez) at the particles through the library,
        with the hand-written adjoint as backward (mesh geometry fixed)."""

        @staticmethod
        def forward(ctx, mesh, x, y, z, q, at_cathode=False):
            ctx.mesh = mesh
            ctx.at_cathode = at_cathode
            ctx.save_for_backward(x, y, z, q)
            return kick(mesh, x.detach(), y.detach(), z.detach(), q.detach(), at_cathode=at_cathode)

        @staticmethod
        def backward(ctx, gx, gy, gz):
            x, y, z, q = ctx.saved_tensors
            dx, dy, dz, dq = kick_adjoint(ctx.mesh, x, y, z, q, gx, gy, gz, at_cathode=ctx.at_cathode)
            return None, dx, dy, dz, dq, None

    return KickFunction


_KICK_FN = None


def kick_autograd(mesh: Mesh3D, x, y, z, q, at_cathode: bool = False):
    """Differentiable kick on CUDA tensors (torch.autograd)."""
    global _KICK_FN
    if _KICK_FN is None:
        _KICK_FN = _make_kick_function()
    return _KICK_FN.apply(mesh, x, y, z, q, at_cathode)


def autotune(mesh: Mesh3D) -> int:
    """Pick the fastest FFT kernel configuration for this mesh's transform
    shape (sc_autotune): 0 = register two-step transforms, 2..5 = Stockham
    transforms with 2**k columns per CTA.  Synchronises."""
    c = C.c_int()
    L.call("sc_autotune", mesh.ptr, _stream(), C.byref(c))
    return int(c.value)


class Batch:
    """Kicks of many independent bunches in one call (sc_batch_kick): each
    bunch has its own mesh; repeated calls with the same particle tensors
    replay a captured CUDA graph.  Output tensors are owned by the batch and
    overwritten by every call with the same inputs."""

    def __init__(self, meshes, nstreams: int = 8):
        self.meshes = list(meshes)  # keep the meshes alive
        arr = (C.c_void_p * len(self.meshes))(*[m.ptr.value for m in self.meshes])
        out = C.c_void_p()
        L.call("sc_batch_create", arr, len(self.meshes), int(nstreams), C.byref(out))
        self._ptr = out
        self._outs = None
        self._key = None

    def __del__(self):
        if getattr(self, "_ptr", None) is not None and self._ptr.value and L._lib is not None:
            L._lib.sc_batch_destroy(self._ptr)
            self._ptr = None

    def set_graph(self, enabled: bool) -> None:
        L.call("sc_batch_set_graph", self._ptr, 1 if enabled else 0)

    def set_staged(self, enabled: bool) -> None:
        """Staged engine on (default) or every bunch on the per-bunch streams."""
        L.call("sc_batch_set_staged", self._ptr, 1 if enabled else 0)

    def set_group_bytes(self, nbytes: int) -> None:
        """Working-set budget of a group of staged bunches (0: one bunch per
        group; a huge value: one group per grid class)."""
        L.call("sc_batch_set_group_bytes", self._ptr, int(nbytes))

    def set_fused_forward(self, enabled: bool) -> None:
        """Staged forward x+y transforms as one fused pass (True) or two."""
        L.call("sc_batch_set_fused_forward", self._ptr, 1 if enabled else 0)

    def autotune(self, xs, ys, zs, qs, at_cathode: bool = False) -> tuple[int, bool]:
        """Times the kick of these bunches for several group budgets and both
        forward-pass forms, keeps the fastest and returns it as
        (group_bytes, fused_forward)."""
        return self.kick(xs, ys, zs, qs, at_cathode=at_cathode, _tune=True)

    @property
    def graph_nodes(self) -> int:
        n = C.c_int64()
        L.call("sc_batch_graph_nodes", self._ptr, C.byref(n))
        return int(n.value)

    @property
    def staged(self) -> tuple[int, int]:
        """(bunches kicked stage by stage, kernel launches of those stages)."""
        k, n = C.c_int(), C.c_int64()
        L.call("sc_batch_staged_count", self._ptr, C.byref(k), C.byref(n))
        return int(k.value), int(n.value)

    def kick(self, xs, ys, zs, qs, at_cathode: bool = False, _tune: bool = False):
        torch = _torch()
        nb = len(self.meshes)
        if not (len(xs) == len(ys) == len(zs) == len(qs) == nb):
            raise SpaceChargeError(f"need particle arrays for each of the {nb} bunches")
        dev = []
        dt = None
        for i in range(nb):
            lens = [_length(a) for a in (xs[i], ys[i], zs[i], qs[i])]
            if not (lens[0] == lens[1] == lens[2] == lens[3]):
                raise SpaceChargeError("Particle coordinate and charge arrays must have the same length.")
            # all bunches take the first bunch's element type; CUDA tensors
            # of that type are used in place (stable pointers: graph replay)
            want = None if dt is None else (torch.float64 if dt == L.SC_F64 else torch.float32)
            t, d = _as_device((xs[i], ys[i], zs[i], qs[i]), dtype=want)
            dt = d
            dev.append(t)
        key = tuple(tuple(t.data_ptr() for t in b) for b in dev)
        if self._outs is None or self._key != key:
            self._outs = [[torch.empty_like(b[0]) for _ in range(3)] for b in dev]
            self._key = key
        self._dev = dev  # keep device copies alive while the graph may read them

        def ptrs(k, src):
            return (C.c_void_p * nb)(*[src[i][k].data_ptr() for i in range(nb)])

        n = (C.c_int64 * nb)(*[int(b[0].numel()) for b in dev])
        args = (ptrs(0, dev), ptrs(1, dev), ptrs(2, dev), ptrs(3, dev), n, dt, 1 if at_cathode else 0,
                ptrs(0, self._outs), ptrs(1, self._outs), ptrs(2, self._outs), _stream())
        if _tune:
            g, f = C.c_int64(), C.c_int()
            L.call("sc_batch_autotune", self._ptr, *args, C.byref(g), C.byref(f))
            return int(g.value), bool(f.value)
        L.call("sc_batch_kick", self._ptr, *args)
        return [tuple(o) for o in self._outs]
