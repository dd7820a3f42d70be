"""
    MeshingGB300

Drop-in GPU back end for Meshing.jl.  Loading this module adds methods of
`Meshing.isosurface` that are more specific than the reference's
(src/marching_cubes.jl:27, src/marching_tetrahedra.jl:129): dense
`Array{T,3}` volumes with `T ∈ {UInt8, Int8, Int16, UInt16, Int32, Int64, Float16, Float32,
Float64}` and
iso / eps / range endpoints of type Float32, Float64 or Int64 run on the GPU through
`libmeshing_gb300.so` (Float16 data with a Float32 or Float64 iso).  Every other
combination (Float16 data with an Int iso, other machine integers, ForwardDiff.Dual,
mixed endpoint types) reaches the reference method through `invoke`, i.e.
ordinary dispatch, not a fallback inside the library.
Results are identical to the reference's: the same element types, vertex
order and 1-based faces.  `NaiveSurfaceNets` (named in the reference's README
but not implemented there) is added with the definition documented in the
library.
"""
module MeshingGB300

using Meshing
import Meshing: isosurface, MarchingCubes, MarchingTetrahedra, AbstractMeshingAlgorithm

export NaiveSurfaceNets, WeldedMarchingCubes

const libmesh = joinpath(@__DIR__, "..", "_build", "libmeshing_gb300.so")

"""
    NaiveSurfaceNets(; iso=0.0)

One vertex per cell straddling `iso` (mean of its edge crossings) and two
triangles per crossed lattice edge, joining the four cells around it.
"""
Base.@kwdef struct NaiveSurfaceNets{T} <: AbstractMeshingAlgorithm
    iso::T = 0.0
end

"""
    WeldedMarchingCubes(; iso=0.0)

Marching Cubes with one vertex per crossed lattice edge (opt-in, not a drop-in
for `MarchingCubes`): vertices numbered when their edge is first met in the
reference's emission order and placed by that cell's `vertex_interp`; faces are
`MarchingCubes`' triangles on those vertices.
"""
Base.@kwdef struct WeldedMarchingCubes{T} <: AbstractMeshingAlgorithm
    iso::T = 0.0
end

# Mirrors mesh_params in include/meshing_gb300.h (C layout).
struct MeshParams
    alg::Int32
    iso_type::Int32
    iso::Float64
    eps_type::Int32
    eps::Float64
    range_type::Int32
    range::NTuple{6,Float64}
end

const DevEl = Union{UInt8,Int8,Int16,UInt16,Int32,Int64,Float16,Float32,Float64}
const DevScalar = Union{Float32,Float64,Int64}

dtcode(::Type{UInt16}) = Int32(1)
dtcode(::Type{Float32}) = Int32(2)
dtcode(::Type{Float64}) = Int32(3)
dtcode(::Type{Int64}) = Int32(4)
dtcode(::Type{Int32}) = Int32(5)
dtcode(::Type{Float16}) = Int32(6)
dtcode(::Type{Int16}) = Int32(7)
dtcode(::Type{Int8}) = Int32(8)
dtcode(::Type{UInt8}) = Int32(9)
# promote(Int, Float16) is Float16: that quotient runs in Float16 arithmetic, left to the reference
device_ok(::Type{T}, ::Type{I}) where {T,I} = !(T === Float16 && I === Int64)
dtcode(::Type) = Int32(0)

# one context per thread: a context is not thread-safe
const CTXS = Dict{Int,Ptr{Cvoid}}()
const CTX_LOCK = ReentrantLock()
function context()
    tid = Threads.threadid()
    lock(CTX_LOCK) do
        get!(CTXS, tid) do
            h = Ref{Ptr{Cvoid}}(C_NULL)
            rc = ccall((:mesh_ctx_create, libmesh), Cint, (Cint, Ref{Ptr{Cvoid}}), 0, h)
            rc == 0 || error("mesh_ctx_create failed: status $rc")
            h[]
        end
    end
end

function check(rc, ctx)
    rc == 0 && return nothing
    msg = unsafe_string(ccall((:mesh_ctx_last_error, libmesh), Cstring, (Ptr{Cvoid},), ctx))
    error("meshing_gb300 status $rc: $msg")
end

supported(X, Y, Z) = (E = typeof(first(X)); E <: DevScalar && typeof(last(X)) == E &&
                      typeof(first(Y)) == E && typeof(last(Y)) == E &&
                      typeof(first(Z)) == E && typeof(last(Z)) == E)

function device_isosurface(sdf::Array{T,3}, alg::Int32, iso, eps, X, Y, Z, ::Type{VT}) where {T,VT}
    E = typeof(first(X))
    p = Ref(MeshParams(alg, dtcode(typeof(iso)), Float64(iso), dtcode(typeof(eps)), Float64(eps), dtcode(E),
                       (Float64(first(X)), Float64(last(X)), Float64(first(Y)), Float64(last(Y)),
                        Float64(first(Z)), Float64(last(Z)))))
    ctx = context()
    nv, nf = Ref{Int64}(0), Ref{Int64}(0)
    nx, ny, nz = size(sdf)
    GC.@preserve sdf begin
        check(ccall((:mesh_count, libmesh), Cint,
                    (Ptr{Cvoid}, Ptr{Cvoid}, Cint, Int64, Int64, Int64, Cint, Ref{MeshParams}, Ref{Int64}, Ref{Int64}),
                    ctx, sdf, dtcode(T), nx, ny, nz, 0, p, nv, nf), ctx)
    end
    vts = Vector{NTuple{3,VT}}(undef, nv[])
    fcs = Vector{NTuple{3,Int}}(undef, nf[])
    GC.@preserve vts fcs begin
        check(ccall((:mesh_fill, libmesh), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Int64}, Cint),
                    ctx, vts, Ptr{Int64}(pointer(fcs)), 0), ctx)
    end
    return vts, fcs
end

function isosurface(sdf::Array{T,3}, method::MarchingCubes{I}, X=-1:1, Y=-1:1, Z=-1:1) where {T<:DevEl,I<:DevScalar}
    (supported(X, Y, Z) && device_ok(T, I)) ||
        return invoke(isosurface, Tuple{AbstractArray{T,3},MarchingCubes,typeof(X),typeof(Y),typeof(Z)},
                      sdf, method, X, Y, Z)
    FT = promote_type(eltype(first(X)), eltype(first(Y)), eltype(first(Z)), T, I)
    device_isosurface(sdf, Int32(0), method.iso, 1e-3, X, Y, Z, float(FT))
end

function isosurface(sdf::Array{T,3}, method::MarchingTetrahedra{I,E}, X=-1:1, Y=-1:1, Z=-1:1) where {T<:DevEl,I<:DevScalar,E<:Union{Float32,Float64}}
    (supported(X, Y, Z) && device_ok(T, I)) ||
        return invoke(isosurface, Tuple{AbstractArray{T,3},MarchingTetrahedra,typeof(X),typeof(Y),typeof(Z)},
                      sdf, method, X, Y, Z)
    FT = promote_type(eltype(first(X)), eltype(first(Y)), eltype(first(Z)), T, I, E)
    device_isosurface(sdf, Int32(1), method.iso, method.eps, X, Y, Z, float(FT))
end

function isosurface(sdf::Array{T,3}, method::NaiveSurfaceNets{I}, X=-1:1, Y=-1:1, Z=-1:1) where {T<:DevEl,I<:DevScalar}
    supported(X, Y, Z) || error("NaiveSurfaceNets: range endpoints must share one of Float32, Float64, Int64")
    device_ok(T, I) || error("NaiveSurfaceNets: Float16 volumes take a Float32 or Float64 iso")
    FT = promote_type(eltype(first(X)), eltype(first(Y)), eltype(first(Z)), T, I)
    device_isosurface(sdf, Int32(2), method.iso, 1e-3, X, Y, Z, float(FT))
end

function isosurface(sdf::Array{T,3}, method::WeldedMarchingCubes{I}, X=-1:1, Y=-1:1, Z=-1:1) where {T<:DevEl,I<:DevScalar}
    supported(X, Y, Z) || error("WeldedMarchingCubes: range endpoints must share one of Float32, Float64, Int64")
    device_ok(T, I) || error("WeldedMarchingCubes: Float16 volumes take a Float32 or Float64 iso")
    FT = promote_type(eltype(first(X)), eltype(first(Y)), eltype(first(Z)), T, I)
    device_isosurface(sdf, Int32(3), method.iso, 1e-3, X, Y, Z, float(FT))
end

end # module
