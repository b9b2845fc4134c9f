"""
    SpaceChargeGB300

Drop-in replacement for SpaceCharge.jl's GPU hot path (src/SpaceCharge.jl:17
exports): `Mesh3D`, `deposit!`, `clear_mesh!`, `solve!`, `interpolate_field`,
backed by libspacecharge_gb300.so (hand-written sm_103a kernels) through
`ccall`.  Particle arrays are `CuArray{Float32}` or `CuArray{Float64}`; work is
enqueued on the task-local CUDA.jl stream, as the reference's kernels are.
A non-zero library status becomes `error(msg)` (an `ErrorException`), as the
reference's argument checks do.
"""
module SpaceChargeGB300

using CUDA
import ChainRulesCore

export Mesh3D, deposit!, clear_mesh!, interpolate_field, solve!, kick, kick!, kick_host, track!, magnetic_field,
       set_kick_mode!, set_fp64_arithmetic!, set_bounds!, refit!, solve_potential

const libsc = normpath(joinpath(@__DIR__, "..", "..", "..", "lib", "libspacecharge_gb300.so"))

const SC_F32 = Cint(0)
const SC_F64 = Cint(1)
const SC_PREC_PLAIN64 = Cint(0)
const SC_PREC_FP64 = Cint(1)
const SC_PREC_MIXED = Cint(2)
const SC_LAYOUT_PACKED = Cint(1)

# include/spacecharge_gb300.h: sc_mesh_info
struct MeshInfo
    grid_size::NTuple{3,Int32}
    precision::Int32
    min_bounds::NTuple{3,Float64}
    max_bounds::NTuple{3,Float64}
    delta::NTuple{3,Float64}
    gamma::Float64
    total_charge::Float64
    efield_layout::Int32
    elem_bytes::Int32
    fft_shape::NTuple{3,Int32}
    device::Int32
end

check(st::Cint) = st == 0 ? nothing :
    error(unsafe_string(ccall((:sc_last_error, libsc), Cstring, ())))

dtype_code(::Type{Float32}) = SC_F32
dtype_code(::Type{Float64}) = SC_F64
stream_ptr() = CUDA.stream().handle

mutable struct Mesh3D{T<:AbstractFloat}
    ptr::Ptr{Cvoid}
    grid_size::NTuple{3,Int}
    min_bounds::NTuple{3,Float64}
    max_bounds::NTuple{3,Float64}
    delta::NTuple{3,Float64}
    gamma::Float64
    total_charge::Float64
    rho::CuArray{T,3}
    efield::AbstractArray{T,4}
end

function _wrap(ptr::Ptr{Cvoid}, ::Type{T}) where {T}
    info = Ref{MeshInfo}()
    check(ccall((:sc_mesh_get_info, libsc), Cint, (Ptr{Cvoid}, Ref{MeshInfo}), ptr, info))
    inf = info[]
    n = Int.(inf.grid_size)
    prho = Ref{Ptr{Cvoid}}(C_NULL)
    pef = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:sc_mesh_rho, libsc), Cint, (Ptr{Cvoid}, Ref{Ptr{Cvoid}}), ptr, prho))
    check(ccall((:sc_mesh_efield, libsc), Cint, (Ptr{Cvoid}, Ref{Ptr{Cvoid}}), ptr, pef))
    rho = unsafe_wrap(CuArray, CuPtr{T}(UInt(prho[])), n)
    efield = if inf.efield_layout == SC_LAYOUT_PACKED
        raw = unsafe_wrap(CuArray, CuPtr{T}(UInt(pef[])), (4, n...))
        PermutedDimsArray(view(raw, 1:3, :, :, :), (2, 3, 4, 1))   # (nx, ny, nz, 3)
    else
        unsafe_wrap(CuArray, CuPtr{T}(UInt(pef[])), (n..., 3))
    end
    m = Mesh3D{T}(ptr, Tuple(n), inf.min_bounds, inf.max_bounds, inf.delta, inf.gamma,
                  inf.total_charge, rho, efield)
    finalizer(m) do mm
        ccall((:sc_mesh_destroy, libsc), Cint, (Ptr{Cvoid},), mm.ptr)
    end
    return m
end

precision_code(::Type{Float64}, p) = p === :plain64 ? SC_PREC_PLAIN64 : SC_PREC_FP64
precision_code(::Type{Float32}, p) = SC_PREC_MIXED
storage_type(code) = code == SC_PREC_MIXED ? Float32 : Float64

# Mesh3D(grid_size, px, py, pz; T, gamma, total_charge), src/mesh.jl:95-174
function Mesh3D(grid_size::NTuple{3,Int}, particles_x::CuArray{P}, particles_y::CuArray{P},
                particles_z::CuArray{P}; T::Type{<:AbstractFloat}=Float64, precision::Symbol=:native,
                gamma::Real=1.0, total_charge::Real=0.0) where {P<:Union{Float32,Float64}}
    if !(length(particles_x) == length(particles_y) == length(particles_z))
        error("Particle coordinate arrays must have the same length.")
    end
    code = precision_code(T, precision)
    out = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:sc_mesh_create_from_particles, libsc), Cint,
                (Ptr{Int32}, CuPtr{P}, CuPtr{P}, CuPtr{P}, Int64, Cint, Float64, Float64, Cint, Ptr{Cvoid},
                 Ref{Ptr{Cvoid}}),
                Int32[grid_size...], particles_x, particles_y, particles_z, length(particles_x), dtype_code(P),
                Float64(gamma), Float64(total_charge), code, stream_ptr(), out))
    return _wrap(out[], storage_type(code))
end

# Mesh3D(grid_size, min_bounds, max_bounds; T, gamma, total_charge), src/mesh.jl:196-238
function Mesh3D(grid_size::NTuple{3,Int}, min_bounds::NTuple{3,Real}, max_bounds::NTuple{3,Real};
                T::Type{<:AbstractFloat}=Float64, precision::Symbol=:native, gamma::Real=1.0,
                total_charge::Real=0.0)
    code = precision_code(T, precision)
    out = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:sc_mesh_create, libsc), Cint,
                (Ptr{Int32}, Ptr{Float64}, Ptr{Float64}, Float64, Float64, Cint, Ref{Ptr{Cvoid}}),
                Int32[grid_size...], Float64[min_bounds...], Float64[max_bounds...], Float64(gamma),
                Float64(total_charge), code, out))
    return _wrap(out[], storage_type(code))
end

# the mesh's bounds after the library changed them
function _sync_bounds!(mesh::Mesh3D)
    info = Ref{MeshInfo}()
    check(ccall((:sc_mesh_get_info, libsc), Cint, (Ptr{Cvoid}, Ref{MeshInfo}), mesh.ptr, info))
    mesh.min_bounds = info[].min_bounds
    mesh.max_bounds = info[].max_bounds
    mesh.delta = info[].delta
    return mesh
end

"""
    set_bounds!(mesh, min_bounds, max_bounds)

New bounds for `mesh`, keeping its grid, fields and workspaces
(sc_mesh_set_bounds; the manual constructor's validation and delta,
src/mesh.jl:206-220).
"""
function set_bounds!(mesh::Mesh3D, min_bounds::NTuple{3,Real}, max_bounds::NTuple{3,Real})
    check(ccall((:sc_mesh_set_bounds, libsc), Cint, (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}), mesh.ptr,
                Float64[min_bounds...], Float64[max_bounds...]))
    return _sync_bounds!(mesh)
end

"""
    refit!(mesh, px, py, pz)

The particle constructor's bounds for these particles (sc_mesh_refit,
src/mesh.jl:95-174).
"""
function refit!(mesh::Mesh3D, px::CuArray{P}, py::CuArray{P}, pz::CuArray{P}) where {P<:Union{Float32,Float64}}
    length(px) == length(py) == length(pz) || error("Particle coordinate arrays must have the same length.")
    check(ccall((:sc_mesh_refit, libsc), Cint, (Ptr{Cvoid}, CuPtr{P}, CuPtr{P}, CuPtr{P}, Int64, Cint, Ptr{Cvoid}),
                mesh.ptr, px, py, pz, length(px), dtype_code(P), stream_ptr()))
    return _sync_bounds!(mesh)
end

# clear_mesh!(mesh), src/deposition.jl:10-12
clear_mesh!(mesh::Mesh3D) =
    check(ccall((:sc_clear_mesh, libsc), Cint, (Ptr{Cvoid}, Ptr{Cvoid}), mesh.ptr, stream_ptr()))

# deposit!(mesh, px, py, pz, pq; clear=true), src/deposition.jl:218-247
function deposit!(mesh::Mesh3D, particles_x::CuArray{P}, particles_y::CuArray{P}, particles_z::CuArray{P},
                  particles_q::CuArray{P}; clear::Bool=true, mode::Symbol=:atomic) where {P<:Union{Float32,Float64}}
    if !(length(particles_x) == length(particles_y) == length(particles_z) == length(particles_q))
        error("Particle coordinate and charge arrays must have the same length.")
    end
    check(ccall((:sc_deposit, libsc), Cint,
                (Ptr{Cvoid}, CuPtr{P}, CuPtr{P}, CuPtr{P}, CuPtr{P}, Int64, Cint, Cint, Cint, Ptr{Cvoid}),
                mesh.ptr, particles_x, particles_y, particles_z, particles_q, length(particles_x),
                dtype_code(P), Cint(clear), deposit_mode_code(mode), stream_ptr()))
end

# include/spacecharge_gb300.h: SC_DEPOSIT_*
const DEPOSIT_MODES = Dict(:atomic => Cint(0), :sorted => Cint(1), :deterministic => Cint(2),
                           :tiled => Cint(3), :vector => Cint(4))
deposit_mode_code(mode::Symbol) =
    get(() -> error("unknown deposit mode $(repr(mode)); expected one of $(sort(collect(keys(DEPOSIT_MODES))))"),
        DEPOSIT_MODES, mode)

"""
    set_kick_mode!(mesh, mode::Symbol)

Deposit mode `kick` uses on this mesh: `:vector` (the default for mixed
meshes), `:atomic` (the default otherwise), `:sorted`, `:deterministic`
(bitwise reproducible) or `:tiled`.
"""
set_kick_mode!(mesh::Mesh3D, mode::Symbol) =
    check(ccall((:sc_mesh_set_kick_mode, libsc), Cint, (Ptr{Cvoid}, Cint), mesh.ptr, deposit_mode_code(mode)))

"""
    set_fp64_arithmetic!(mesh, mode::Symbol)

`Float64` meshes: `:fp64` (the default) runs the kick in FP64; `:df32` runs
the atomic deposit's weights, the x, y and (free-space) z transform passes and
the interpolation in double-FP32 (pairs of `Float32`, 48-bit significands,
about 1e-14 of the fields' maximum), off the GPU's FP64 units.
"""
set_fp64_arithmetic!(mesh::Mesh3D, mode::Symbol) =
    check(ccall((:sc_mesh_set_fp64_arithmetic, libsc), Cint, (Ptr{Cvoid}, Cint), mesh.ptr,
                mode === :fp64 ? Cint(0) : mode === :df32 ? Cint(1) : throw(ArgumentError("mode: :fp64 or :df32"))))

# solve!(mesh; at_cathode=false), src/solvers/free_space.jl:14-47
solve!(mesh::Mesh3D; at_cathode::Bool=false) =
    check(ccall((:sc_solve, libsc), Cint, (Ptr{Cvoid}, Cint, Ptr{Cvoid}), mesh.ptr, Cint(at_cathode),
                stream_ptr()))

# solve_potential(mesh; at_cathode=false) -> phi::CuArray{T,3}: the scalar
# potential of the deposited charge with potential_green_function
# (src/green_functions.jl:13-22, defined but not called by the reference)
function solve_potential(mesh::Mesh3D{T}; at_cathode::Bool=false) where {T}
    phi = CuArray{T}(undef, mesh.grid_size...)
    check(ccall((:sc_solve_potential, libsc), Cint, (Ptr{Cvoid}, Cint, CuPtr{T}, Ptr{Cvoid}), mesh.ptr,
                Cint(at_cathode), pointer(phi), stream_ptr()))
    return phi
end

# interpolate_field(mesh, px, py, pz) -> (Ex, Ey, Ez), src/interpolation.jl:100-128
function interpolate_field(mesh::Mesh3D, particles_x::CuArray{P}, particles_y::CuArray{P},
                           particles_z::CuArray{P}) where {P<:Union{Float32,Float64}}
    Ex = similar(particles_x); Ey = similar(particles_x); Ez = similar(particles_x)
    check(ccall((:sc_interpolate_field, libsc), Cint,
                (Ptr{Cvoid}, CuPtr{P}, CuPtr{P}, CuPtr{P}, Int64, Cint, CuPtr{P}, CuPtr{P}, CuPtr{P}, Ptr{Cvoid}),
                mesh.ptr, particles_x, particles_y, particles_z, length(particles_x), dtype_code(P),
                Ex, Ey, Ez, stream_ptr()))
    return Ex, Ey, Ez
end

"""
    kick(mesh, px, py, pz, pq; at_cathode=false) -> (Ex, Ey, Ez)

deposit! + solve! + interpolate_field in one library call.  Differentiable:
the `rrule` below runs the hand-written adjoint (sc_kick_adjoint) for
d(loss)/d(px, py, pz, pq) with the mesh geometry held fixed.
"""
function kick(mesh::Mesh3D, px::CuArray{P}, py::CuArray{P}, pz::CuArray{P}, pq::CuArray{P};
              at_cathode::Bool=false) where {P<:Union{Float32,Float64}}
    Ex = similar(px); Ey = similar(px); Ez = similar(px)
    return kick!(Ex, Ey, Ez, mesh, px, py, pz, pq; at_cathode=at_cathode)
end

"""
    kick!(Ex, Ey, Ez, mesh, px, py, pz, pq; at_cathode=false) -> (Ex, Ey, Ez)

`kick` into caller-owned field arrays.  Repeated calls with the same arrays
replay a CUDA graph of the kick (sc_kick), which `kick`'s fresh outputs
rule out.
"""
function kick!(Ex::CuArray{P}, Ey::CuArray{P}, Ez::CuArray{P}, mesh::Mesh3D, px::CuArray{P}, py::CuArray{P},
               pz::CuArray{P}, pq::CuArray{P}; at_cathode::Bool=false) where {P<:Union{Float32,Float64}}
    length(px) == length(py) == length(pz) == length(pq) == length(Ex) == length(Ey) == length(Ez) ||
        error("Particle coordinate and charge arrays must have the same length.")
    check(ccall((:sc_kick, libsc), Cint,
                (Ptr{Cvoid}, CuPtr{P}, CuPtr{P}, CuPtr{P}, CuPtr{P}, Int64, Cint, Cint, CuPtr{P}, CuPtr{P},
                 CuPtr{P}, Ptr{Cvoid}),
                mesh.ptr, px, py, pz, pq, length(px), dtype_code(P), Cint(at_cathode), Ex, Ey, Ez, stream_ptr()))
    return Ex, Ey, Ez
end

function ChainRulesCore.rrule(::typeof(kick), mesh::Mesh3D, px::CuArray{P}, py::CuArray{P}, pz::CuArray{P},
                              pq::CuArray{P}; at_cathode::Bool=false) where {P<:Union{Float32,Float64}}
    out = kick(mesh, px, py, pz, pq; at_cathode=at_cathode)
    function kick_pullback(Δ)
        gx, gy, gz = map(d -> d isa ChainRulesCore.AbstractZero ? CUDA.zeros(P, length(px)) : CuArray{P}(d),
                         ChainRulesCore.unthunk(Δ))
        dx = similar(px); dy = similar(px); dz = similar(px); dq = similar(px)
        check(ccall((:sc_kick_adjoint, libsc), Cint,
                    (Ptr{Cvoid}, CuPtr{P}, CuPtr{P}, CuPtr{P}, CuPtr{P}, Int64, Cint, Cint, CuPtr{P}, CuPtr{P},
                     CuPtr{P}, Ptr{Cvoid}, CuPtr{P}, CuPtr{P}, CuPtr{P}, CuPtr{P}, Ptr{Cvoid}),
                    mesh.ptr, px, py, pz, pq, length(px), dtype_code(P), Cint(at_cathode), gx, gy, gz, C_NULL,
                    dx, dy, dz, dq, stream_ptr()))
        return (ChainRulesCore.NoTangent(), ChainRulesCore.NoTangent(), dx, dy, dz, dq)
    end
    return out, kick_pullback
end

"""
    kick_host(mesh, px, py, pz, pq; at_cathode=false) -> (Ex, Ey, Ez)

`kick` for particles in host memory (sc_kick_host): the library streams the
arrays to the GPU in chunks, overlapping the copies with the deposit and the
gather.  Page-locked arrays (`CUDA.Mem.pin`) give the overlap.
"""
function kick_host(mesh::Mesh3D, px::Vector{P}, py::Vector{P}, pz::Vector{P}, pq::Vector{P};
                   at_cathode::Bool=false) where {P<:Union{Float32,Float64}}
    length(px) == length(py) == length(pz) == length(pq) ||
        error("Particle coordinate and charge arrays must have the same length.")
    Ex = similar(px); Ey = similar(px); Ez = similar(px)
    check(ccall((:sc_kick_host, libsc), Cint,
                (Ptr{Cvoid}, Ptr{P}, Ptr{P}, Ptr{P}, Ptr{P}, Int64, Cint, Cint, Ptr{P}, Ptr{P}, Ptr{P}, Ptr{Cvoid}),
                mesh.ptr, px, py, pz, pq, length(px), dtype_code(P), Cint(at_cathode), Ex, Ey, Ez, stream_ptr()))
    CUDA.synchronize()
    return Ex, Ey, Ez
end

"""
    track!(mesh, x, y, z, ux, uy, uz, q; dt, qm, steps=1, refit=true, at_cathode=false)

`steps` tracking steps of the bunch in its own field (sc_track): refit the
mesh bounds, kick, B = (beta/c) z x E, one relativistic Boris step of
u = gamma*beta and the positions over `dt` seconds for charge/mass `qm`.
"""
function track!(mesh::Mesh3D, x::CuArray{P}, y::CuArray{P}, z::CuArray{P}, ux::CuArray{P}, uy::CuArray{P},
                uz::CuArray{P}, q::CuArray{P}; dt::Real, qm::Real, steps::Integer=1, refit::Bool=true,
                at_cathode::Bool=false) where {P<:Union{Float32,Float64}}
    check(ccall((:sc_track, libsc), Cint,
                (Ptr{Cvoid}, CuPtr{P}, CuPtr{P}, CuPtr{P}, CuPtr{P}, CuPtr{P}, CuPtr{P}, CuPtr{P}, Int64, Cint,
                 Cdouble, Cdouble, Cint, Cint, Cint, Ptr{Cvoid}),
                mesh.ptr, x, y, z, ux, uy, uz, q, length(x), dtype_code(P), Float64(dt), Float64(qm), Cint(steps),
                Cint(refit), Cint(at_cathode), stream_ptr()))
    refit && _sync_bounds!(mesh)
    return nothing
end

"""
    magnetic_field(mesh, Ex, Ey) -> (Bx, By)

B = (beta/c) z x E of a bunch moving along +z at the mesh's gamma.
"""
function magnetic_field(mesh::Mesh3D, Ex::CuArray{P}, Ey::CuArray{P}) where {P<:Union{Float32,Float64}}
    Bx = similar(Ex); By = similar(Ex)
    check(ccall((:sc_magnetic_field, libsc), Cint,
                (Ptr{Cvoid}, CuPtr{P}, CuPtr{P}, Int64, Cint, CuPtr{P}, CuPtr{P}, Ptr{Cvoid}),
                mesh.ptr, Ex, Ey, length(Ex), dtype_code(P), Bx, By, stream_ptr()))
    return Bx, By
end

# Host arrays (where the reference would run on its CPU backend): the
# particles are copied to the device, the work runs there, and field outputs
# come back as host arrays.
Mesh3D(grid_size::NTuple{3,Int}, px::Vector{P}, py::Vector{P}, pz::Vector{P};
       kw...) where {P<:Union{Float32,Float64}} = Mesh3D(grid_size, CuArray(px), CuArray(py), CuArray(pz); kw...)

deposit!(mesh::Mesh3D, px::Vector{P}, py::Vector{P}, pz::Vector{P}, pq::Vector{P};
         kw...) where {P<:Union{Float32,Float64}} =
    deposit!(mesh, CuArray(px), CuArray(py), CuArray(pz), CuArray(pq); kw...)

interpolate_field(mesh::Mesh3D, px::Vector{P}, py::Vector{P}, pz::Vector{P}) where {P<:Union{Float32,Float64}} =
    map(Array, interpolate_field(mesh, CuArray(px), CuArray(py), CuArray(pz)))

kick(mesh::Mesh3D, px::Vector{P}, py::Vector{P}, pz::Vector{P}, pq::Vector{P};
     at_cathode::Bool=false) where {P<:Union{Float32,Float64}} = kick_host(mesh, px, py, pz, pq; at_cathode=at_cathode)

function Base.show(io::IO, mesh::Mesh3D{T}) where {T}  # src/mesh.jl:240-246
    nx, ny, nz = mesh.grid_size
    lo, hi = mesh.min_bounds, mesh.max_bounds
    print(io, "Mesh3D{$T, CuArray} ($(nx)x$(ny)x$(nz)) bounds=[($(lo[1]),$(lo[2]),$(lo[3])), " *
              "($(hi[1]),$(hi[2]),$(hi[3]))] gamma=$(mesh.gamma)")
end

end # module
