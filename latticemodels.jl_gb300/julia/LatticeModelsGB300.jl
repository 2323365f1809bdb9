# LatticeModelsGB300 — Julia glue for the GB300 evolution backend (liblmgpu.so).
#
# Adds `ChebyshevGPU <: LatticeModels.EvolutionSolver` and a lazy device Hamiltonian so that
#     Evolution(ChebyshevGPU(tol=1e-12), t -> gpu_tightbinding(l; field=PointFlux(B(t), p)), P0)
# runs the reference's own `Evolution` driver (src/evolution.jl:183-298) on the GPU.
# Every call goes through the C ABI declared in include/lmgpu.h.
module LatticeModelsGB300

using LatticeModels
import LatticeModels: EvolutionSolver, update_solver!, step!, evolution_cache, localdensity

const LIB = get(ENV, "LMGPU_LIB", joinpath(@__DIR__, "..", "lmgpu", "liblmgpu.so"))

const LM_C64 = Cint(0)
const LM_C32 = Cint(1)
const LM_KETS = Cint(0)
const LM_DENSITY = Cint(1)
const LM_FIELD_LANDAU = Cint(1)
const LM_FIELD_SYMMETRIC = Cint(2)
const LM_FIELD_POINTFLUX_AXIAL = Cint(3)
const LM_FIELD_POINTFLUX_SINGULAR = Cint(4)

struct LMError <: Exception
    code::Cint
    msg::String
end

function check(rc::Cint, ctx::Ptr{Cvoid})
    rc == 0 && return nothing
    msg = ctx == C_NULL ? "" : unsafe_string(ccall((:lm_last_error, LIB), Cstring, (Ptr{Cvoid},), ctx))
    throw(LMError(rc, msg))
end

# ---- context -------------------------------------------------------------------------------
mutable struct Context
    handle::Ptr{Cvoid}
    function Context(device::Integer=0)
        h = Ref{Ptr{Cvoid}}(C_NULL)
        check(ccall((:lm_ctx_create, LIB), Cint, (Cint, Ref{Ptr{Cvoid}}), device, h), C_NULL)
        c = new(h[])
        finalizer(c -> ccall((:lm_ctx_destroy, LIB), Cint, (Ptr{Cvoid},), c.handle), c)
        return c
    end
end
const DEFAULT = Ref{Union{Nothing,Context}}(nothing)
default_context() = something(DEFAULT[], (DEFAULT[] = Context(0)))

# ---- lattice (SquareLattice(Lx, Ly; boundaries), src/zoo/lattices.jl:131) -------------------
mutable struct DeviceLattice
    ctx::Context
    handle::Ptr{Cvoid}
    Lx::Int
    Ly::Int
end
function DeviceLattice(Lx, Ly; periodic=(false, false), twist=(0.0, 0.0), ctx=default_context())
    h = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:lm_lattice_square, LIB), Cint,
                (Ptr{Cvoid}, Int64, Int64, Cint, Cint, Cdouble, Cdouble, Ref{Ptr{Cvoid}}),
                ctx.handle, Lx, Ly, periodic[1], periodic[2], twist[1], twist[2], h), ctx.handle)
    l = DeviceLattice(ctx, h[], Lx, Ly)
    finalizer(l -> ccall((:lm_lattice_destroy, LIB), Cint, (Ptr{Cvoid},), l.handle), l)
    return l
end

# ---- lazy device Hamiltonian: the `.data` of the Hamiltonian h(t) returns --------------------
# Holds the parameters; `==` compares them, which keeps CachedExp's `mat == old` cache rule
# (src/evolution.jl:87) meaningful for the GPU solver too.
mutable struct DeviceHamiltonian <: AbstractMatrix{ComplexF64}
    lat::DeviceLattice
    handle::Ptr{Cvoid}
    kinds::Vector{Cint}
    amplitudes::Vector{Float64}
    onsite::Union{Nothing,Vector{Float64}}
end
Base.size(H::DeviceHamiltonian) = (H.lat.Lx * H.lat.Ly, H.lat.Lx * H.lat.Ly)
Base.getindex(::DeviceHamiltonian, ::Int, ::Int) =
    throw(ArgumentError("DeviceHamiltonian lives on the GPU; use lm_ham_csc to download it"))
Base.:(==)(a::DeviceHamiltonian, b::DeviceHamiltonian) =
    a.handle == b.handle && a.amplitudes == b.amplitudes && a.onsite == b.onsite

field_components(::LatticeModels.NoField) = Tuple{Cint,Float64,Float64,Float64}[]
field_components(f::LandauGauge) = [(LM_FIELD_LANDAU, 0.0, 0.0, f.B)]
field_components(f::SymmetricGauge) = [(LM_FIELD_SYMMETRIC, 0.0, 0.0, f.B)]
field_components(f::PointFlux{:axial}) = [(LM_FIELD_POINTFLUX_AXIAL, f.point..., f.flux)]
field_components(f::PointFlux{:singular}) = [(LM_FIELD_POINTFLUX_SINGULAR, f.point..., f.flux)]
field_components(f::LatticeModels.FieldSum) = reduce(vcat, map(field_components, f.fields))

# tightbinding_hamiltonian(l; t1, field) with on-device assembly
# (src/operators/constructoperator.jl:190-194)
function gpu_tightbinding(lat::DeviceLattice, onsite=nothing; t1=1.0, field=LatticeModels.NoField())
    comps = field_components(field)
    h = Ref{Ptr{Cvoid}}(C_NULL)
    ctx = lat.ctx.handle
    check(ccall((:lm_ham_create, LIB), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Cdouble, Ref{Ptr{Cvoid}}),
                ctx, lat.handle, t1, h), ctx)
    for (kind, px, py, _) in comps
        idx = Ref{Cint}(0)
        check(ccall((:lm_ham_add_field, LIB), Cint, (Ptr{Cvoid}, Cint, Cdouble, Cdouble, Cint, Ref{Cint}),
                    h[], kind, px, py, 1, idx), ctx)
    end
    if onsite !== nothing
        v = Vector{Float64}(onsite)
        check(ccall((:lm_ham_set_onsite, LIB), Cint, (Ptr{Cvoid}, Ptr{Float64}), h[], v), ctx)
    end
    H = DeviceHamiltonian(lat, h[], [c[1] for c in comps], [c[4] for c in comps],
                          onsite === nothing ? nothing : Vector{Float64}(onsite))
    finalizer(H -> ccall((:lm_ham_destroy, LIB), Cint, (Ptr{Cvoid},), H.handle), H)
    assemble!(H)
    return H
end

assemble!(H::DeviceHamiltonian) =
    check(ccall((:lm_ham_assemble, LIB), Cint, (Ptr{Cvoid}, Ptr{Float64}, Cint),
                H.handle, H.amplitudes, length(H.amplitudes)), H.lat.ctx.handle)

# ---- device states (the `.data` of Ket/Operator states) -------------------------------------
mutable struct DeviceState <: AbstractMatrix{ComplexF64}
    lat::DeviceLattice
    handle::Ptr{Cvoid}
    n::Int
    m::Int
    kind::Cint
    precision::Cint
end
Base.size(s::DeviceState) = (s.n, s.m)
function DeviceState(lat::DeviceLattice, data::AbstractMatrix; density=false, precision=LM_C64)
    n, m = size(data)
    h = Ref{Ptr{Cvoid}}(C_NULL)
    ctx = lat.ctx.handle
    kind = density ? LM_DENSITY : LM_KETS
    check(ccall((:lm_state_create, LIB), Cint, (Ptr{Cvoid}, Int64, Int64, Cint, Cint, Ref{Ptr{Cvoid}}),
                ctx, n, m, kind, precision, h), ctx)
    host = precision == LM_C64 ? Matrix{ComplexF64}(data) : Matrix{ComplexF32}(data)
    check(ccall((:lm_state_upload, LIB), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Int64), h[], host, n), ctx)
    s = DeviceState(lat, h[], n, m, kind, precision)
    finalizer(s -> ccall((:lm_state_destroy, LIB), Cint, (Ptr{Cvoid},), s.handle), s)
    return s
end
function Base.copy(s::DeviceState)
    h = Ref{Ptr{Cvoid}}(C_NULL)
    ctx = s.lat.ctx.handle
    check(ccall((:lm_state_create, LIB), Cint, (Ptr{Cvoid}, Int64, Int64, Cint, Cint, Ref{Ptr{Cvoid}}),
                ctx, s.n, s.m, s.kind, s.precision, h), ctx)
    check(ccall((:lm_state_copy, LIB), Cint, (Ptr{Cvoid}, Ptr{Cvoid}), h[], s.handle), ctx)
    c = DeviceState(s.lat, h[], s.n, s.m, s.kind, s.precision)
    finalizer(c -> ccall((:lm_state_destroy, LIB), Cint, (Ptr{Cvoid},), c.handle), c)
    return c
end
function Base.Array(s::DeviceState)
    out = s.precision == LM_C64 ? Matrix{ComplexF64}(undef, s.n, s.m) : Matrix{ComplexF32}(undef, s.n, s.m)
    check(ccall((:lm_state_download, LIB), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Int64), s.handle, out, s.n),
          s.lat.ctx.handle)
    return out
end

# ---- the EvolutionSolver plugin (src/evolution.jl:5-33) --------------------------------------
mutable struct ChebyshevGPU <: EvolutionSolver
    ctx::Context
    handle::Ptr{Cvoid}
end
function ChebyshevGPU(_ham=nothing; tol=1e-12, ctx=default_context())
    h = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:lm_solver_create, LIB), Cint, (Ptr{Cvoid}, Cdouble, Ref{Ptr{Cvoid}}), ctx.handle, tol, h),
          ctx.handle)
    s = ChebyshevGPU(ctx, h[])
    finalizer(s -> ccall((:lm_solver_destroy, LIB), Cint, (Ptr{Cvoid},), s.handle), s)
    return s
end

function update_solver!(s::ChebyshevGPU, H::DeviceHamiltonian, dt, force=false)
    assemble!(H)
    check(ccall((:lm_solver_update, LIB), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Cdouble, Cint),
                s.handle, H.handle, dt, force), s.ctx.handle)
end
step!(s::ChebyshevGPU, st::DeviceState, _cache) =
    check(ccall((:lm_solver_step, LIB), Cint, (Ptr{Cvoid}, Ptr{Cvoid}), s.handle, st.handle), s.ctx.handle)
evolution_cache(::ChebyshevGPU, ::DeviceState) = nothing

# ---- readouts ---------------------------------------------------------------------------------
function localdensity(st::DeviceState)
    out = Vector{Float64}(undef, st.n)
    check(ccall((:lm_localdensity, LIB), Cint, (Ptr{Cvoid}, Ptr{Float64}), st.handle, out), st.lat.ctx.handle)
    return out
end
function bond_currents(H::DeviceHamiltonian, st::DeviceState)
    nb = ccall((:lm_lattice_nbonds, LIB), Int64, (Ptr{Cvoid},), H.lat.handle)
    out = Vector{Float64}(undef, nb)
    check(ccall((:lm_bond_currents, LIB), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Float64}), H.handle, st.handle, out),
          st.lat.ctx.handle)
    return out
end

export ChebyshevGPU, DeviceLattice, DeviceState, gpu_tightbinding, bond_currents

end # module
