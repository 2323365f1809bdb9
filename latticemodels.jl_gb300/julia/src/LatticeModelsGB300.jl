# LatticeModelsGB300 — Julia glue for the GB300 evolution backend (liblmgpu.so).
#
# A drop-in for LatticeModels.jl's time-evolution path.  The reference README example runs
# with only the builder and solver arguments added:
#
#     l = SquareLattice(10, 10)
#     h(B) = tightbinding_hamiltonian(GPUBuilder, l, field=PointFlux(B, (5.5, 5.5)))
#     P_0 = densitymatrix(h(0), mu = 0)
#     ev = Evolution(ChebyshevGPU, t -> h(0.2 * min(t, τ) / τ), P_0)
#     for (P, H, t) in ev(0:0.1:2τ)
#         localdensity(P)            # a LatticeValue, read out on the device
#         DensityCurrents(H, P)      # lazy; Currents(...) materialises it from the device bonds
#     end
#
# `GPUBuilder` plugs into the reference's builder hook `construct_operator(BT::Type, sys, ...)`
# (src/operators/constructoperator.jl:136), so `tightbinding_hamiltonian` returns the
# reference's own `Hamiltonian` whose `.data` is a lazy `DeviceHamiltonian`.  `densitymatrix`
# on such a Hamiltonian returns an `Operator` whose `.data` is a `DeviceState`; the reference's
# `Evolution` copies it (device to device) and calls the `ChebyshevGPU` plugin methods
# `update_solver!`/`step!` (src/evolution.jl:5-33, :238-250).  Every call goes through the C ABI
# declared in include/lmgpu.h.
module LatticeModelsGB300

using LatticeModels
import LatticeModels: EvolutionSolver, update_solver!, step!, evolution_cache, localdensity, densitymatrix,
                      construct_operator, Currents, DensityCurrents
import QuantumOpticsBase
import LinearAlgebra
using SparseArrays: SparseMatrixCSC, nnz, nzrange, rowvals, sparse

const LIB = get(ENV, "LMGPU_LIB", joinpath(@__DIR__, "..", "..", "lmgpu", "liblmgpu.so"))

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
# A light value (geometry, t1, field components and amplitudes, on-site term).  Calling h(t)
# every step, as `Evolution(t -> h(t), P_0)` does, only makes a new value: the device tables
# (one lm_ham per lattice, t1 and field structure) are cached and re-assembled on the GPU when
# the amplitudes or the on-site term change.  `==` compares the parameters, which keeps
# CachedExp's `mat == old` cache rule (src/evolution.jl:87) meaningful for the GPU solver too.
mutable struct DeviceHamSlot
    handle::Ptr{Cvoid}
    ctx::Context
    assembled::Any        # (amplitudes, onsite) last assembled, compared by identity
end
const _HAMS = Dict{Any,DeviceHamSlot}()

struct DeviceHamiltonian <: AbstractMatrix{ComplexF64}
    lat::DeviceLattice
    t1::Float64
    comps::Vector{Tuple{Cint,Float64,Float64}}   # (kind, point x, point y) per field component
    amplitudes::Vector{Float64}
    onsite::Union{Nothing,Vector{Float64}}
    auto_pbc::Bool
end
Base.size(H::DeviceHamiltonian) = (H.lat.Lx * H.lat.Ly, H.lat.Lx * H.lat.Ly)
Base.getindex(::DeviceHamiltonian, ::Int, ::Int) =
    throw(ArgumentError("DeviceHamiltonian lives on the GPU; use lm_ham_csc to download it"))
Base.:(==)(a::DeviceHamiltonian, b::DeviceHamiltonian) =
    a.lat === b.lat && a.t1 == b.t1 && a.comps == b.comps && a.amplitudes == b.amplitudes &&
    a.onsite == b.onsite && a.auto_pbc == b.auto_pbc

field_components(::LatticeModels.NoField) = Tuple{Cint,Float64,Float64,Float64}[]
field_components(f::LandauGauge) = [(LM_FIELD_LANDAU, 0.0, 0.0, f.B)]
field_components(f::SymmetricGauge) = [(LM_FIELD_SYMMETRIC, 0.0, 0.0, f.B)]
field_components(f::PointFlux{:axial}) = [(LM_FIELD_POINTFLUX_AXIAL, f.point..., f.flux)]
field_components(f::PointFlux{:singular}) = [(LM_FIELD_POINTFLUX_SINGULAR, f.point..., f.flux)]
field_components(f::LatticeModels.FieldSum) = reduce(vcat, map(field_components, f.fields))

# tightbinding_hamiltonian(l; t1, field) with on-device assembly
# (src/operators/constructoperator.jl:190-194)
function gpu_tightbinding(lat::DeviceLattice, onsite=nothing; t1=1.0, field=LatticeModels.NoField(),
                          auto_pbc=true)
    comps = field_components(field)
    return DeviceHamiltonian(lat, Float64(t1), [(c[1], c[2], c[3]) for c in comps], [c[4] for c in comps],
                             onsite === nothing ? nothing : Vector{Float64}(onsite), auto_pbc)
end

function _new_slot(H::DeviceHamiltonian)
    h = Ref{Ptr{Cvoid}}(C_NULL)
    ctx = H.lat.ctx.handle
    check(ccall((:lm_ham_create, LIB), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Cdouble, Ref{Ptr{Cvoid}}),
                ctx, H.lat.handle, H.t1, h), ctx)
    for (kind, px, py) in H.comps
        idx = Ref{Cint}(0)
        check(ccall((:lm_ham_add_field, LIB), Cint, (Ptr{Cvoid}, Cint, Cdouble, Cdouble, Cint, Ref{Cint}),
                    h[], kind, px, py, H.auto_pbc, idx), ctx)
    end
    s = DeviceHamSlot(h[], H.lat.ctx, nothing)
    finalizer(s -> ccall((:lm_ham_destroy, LIB), Cint, (Ptr{Cvoid},), s.handle), s)
    return s
end

function _assemble!(slot::DeviceHamSlot, H::DeviceHamiltonian)
    if slot.assembled === nothing || slot.assembled[1] !== H.amplitudes || slot.assembled[2] !== H.onsite
        ctx = H.lat.ctx.handle
        check(ccall((:lm_ham_set_onsite, LIB), Cint, (Ptr{Cvoid}, Ptr{Float64}), slot.handle,
                    H.onsite === nothing ? Ptr{Float64}(C_NULL) : H.onsite), ctx)
        check(ccall((:lm_ham_assemble, LIB), Cint, (Ptr{Cvoid}, Ptr{Float64}, Cint),
                    slot.handle, H.amplitudes, length(H.amplitudes)), ctx)
        slot.assembled = (H.amplitudes, H.onsite)
    end
    return slot.handle
end

# The lm_ham of H, assembled with H's amplitudes and on-site term (shared through the cache:
# valid until another Hamiltonian of the same structure is assembled).
handle(H::DeviceHamiltonian) = _assemble!(get!(() -> _new_slot(H), _HAMS, (H.lat, H.t1, H.comps, H.auto_pbc)), H)

# An lm_ham owned by the caller (not shared), assembled once: for batches, which keep it.
private_slot(H::DeviceHamiltonian) = (s = _new_slot(H); _assemble!(s, H); s)

# ---- the drop-in builder: tightbinding_hamiltonian(GPUBuilder, l; t1, field) -----------------
"""
    GPUBuilder

Builder type for the reference's Hamiltonian constructors.  `tightbinding_hamiltonian(GPUBuilder,
l, [V]; t1, field, auto_pbc_field)` and `construct_hamiltonian(GPUBuilder, l, terms...)` return
the reference's `Hamiltonian` with a `DeviceHamiltonian` as `.data`: H(t) is assembled on the
GPU (src/operators/constructoperator.jl:136-156, :190-194).  Terms: nearest-neighbour hopping
`t1 => NearestNeighbor(1)` (t2 = t3 = 0), on-site `LatticeValue`s and numbers; `l` is a 2D
`SquareLattice` with open, periodic or twisted boundaries.  Other lattices and models go
through `GPUSparseHamiltonian` (their `construct_operator` CSC).
"""
struct GPUBuilder end

const _LATTICES = IdDict{Any,DeviceLattice}()   # one device geometry per reference lattice

_tvec(tr::LatticeModels.BravaisTranslation) = Vector{Float64}(tr.translate_uc)
_tvec(tr::LatticeModels.Translation) = Vector{Float64}(tr.R)

# (Lx, Ly, periodic, twist) of a reference SquareLattice(Lx, Ly; boundaries) whose sites are in
# the reference's order, index = (x - 1) Ly + y (src/lattices/bravais/unitcell.jl:126-132).
function square_geometry(l)
    LatticeModels.checklatticetype(l, LatticeModels.SquareLattice{2})
    xs, ys = LatticeModels.coordvalues(l)
    x, y = xs.values, ys.values
    Lx = round(Int, maximum(x) - minimum(x)) + 1
    Ly = round(Int, maximum(y) - minimum(y)) + 1
    (length(l) == Lx * Ly && x == repeat(minimum(x) .+ (0:Lx-1), inner=Ly) &&
     y == repeat(minimum(y) .+ (0:Ly-1), outer=Lx)) ||
        throw(ArgumentError("GPUBuilder needs a full rectangular SquareLattice(Lx, Ly)"))
    periodic = [false, false]
    twist = [0.0, 0.0]
    for b in LatticeModels.getboundaries(l).boundaries
        b isa LatticeModels.TwistedBoundary ||
            throw(ArgumentError("GPUBuilder: only periodic or twisted boundaries, not $(typeof(b))"))
        v = _tvec(b.translation)
        ax = findfirst(!iszero, v)
        (count(!iszero, v) == 1 && abs(v[ax]) == (Lx, Ly)[ax]) ||
            throw(ArgumentError("GPUBuilder: boundary translation $v is not a lattice axis"))
        periodic[ax] = true
        twist[ax] = v[ax] > 0 ? b.Θ : -b.Θ
    end
    return Lx, Ly, (periodic[1], periodic[2]), (twist[1], twist[2])
end

function device_lattice(l; ctx=default_context())
    get!(_LATTICES, l) do
        Lx, Ly, periodic, twist = square_geometry(l)
        DeviceLattice(Lx, Ly; periodic=periodic, twist=twist, ctx=ctx)
    end
end

function LatticeModels.construct_operator(::Type{GPUBuilder}, sys::LatticeModels.System, args...;
                                          field=LatticeModels.NoField(), auto_pbc_field=true, kw...)
    smp = LatticeModels.sample(sys)
    LatticeModels.hasinternal(smp) &&
        throw(ArgumentError("GPUBuilder: internal degrees of freedom go through GPUSparseHamiltonian"))
    l = LatticeModels.lattice(smp)
    t1 = 0.0
    onsite = nothing
    for arg in args
        amp, onlat = arg isa Pair ? (arg[1], arg[2]) : (1, arg)
        amp isa Number || throw(ArgumentError("GPUBuilder: operator-valued terms need GPUSparseHamiltonian"))
        iszero(amp) && continue   # zero terms are skipped (src/operators/constructoperator.jl:50)
        if onlat isa LatticeModels.NearestNeighbor{1}
            t1 += real(amp)
        elseif onlat isa LatticeModels.NearestNeighbor
            throw(ArgumentError("GPUBuilder: only nearest-neighbour hopping (t2 = t3 = 0)"))
        elseif onlat isa LatticeModels.LatticeValue
            onsite = something(onsite, zeros(length(l)))
            onsite .+= real(amp) .* onlat.values
        elseif onlat isa Number
            onsite = something(onsite, zeros(length(l)))
            onsite .+= real(amp * onlat)
        else
            throw(ArgumentError("GPUBuilder: cannot interpret $(typeof(onlat)) as a term"))
        end
    end
    H = gpu_tightbinding(device_lattice(l), onsite; t1=t1, field=field, auto_pbc=auto_pbc_field)
    return QuantumOpticsBase.Operator(LatticeModels.basis(sys), H)
end

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

# A device ket: the `.data` of a reference `Ket` (an AbstractVector, as QuantumOpticsBase
# requires) backed by an N x 1 device state.
struct DeviceVector <: AbstractVector{ComplexF64}
    st::DeviceState
end
Base.size(v::DeviceVector) = (v.st.n,)
Base.getindex(::DeviceVector, ::Int) =
    throw(ArgumentError("DeviceVector lives on the GPU; use Array(v) to download it"))
Base.copy(v::DeviceVector) = DeviceVector(copy(v.st))
Base.Array(v::DeviceVector) = vec(Array(v.st))

# A context-only geometry handle for states on lattices the square-lattice path does not know
const _CTX_LATTICES = IdDict{Context,DeviceLattice}()
context_lattice(ctx::Context) = get!(() -> DeviceLattice(ctx, C_NULL, 0, 0), _CTX_LATTICES, ctx)

"""
    to_device(state; precision=LM_C64)

A copy of a reference `Ket` or density-matrix `Operator` whose `.data` lives on the GPU, for
`Evolution(ChebyshevGPU, h, to_device(psi))`.  `Array(state.data)` downloads it.
"""
function to_device(psi::QuantumOpticsBase.Ket; precision=LM_C64, ctx=default_context())
    lat = _state_lattice(psi, ctx)
    return QuantumOpticsBase.Ket(QuantumOpticsBase.basis(psi),
                                 DeviceVector(DeviceState(lat, reshape(psi.data, :, 1); precision=precision)))
end
function to_device(P::QuantumOpticsBase.Operator; precision=LM_C64, ctx=default_context())
    lat = _state_lattice(P, ctx)
    return QuantumOpticsBase.Operator(P.basis_l, P.basis_r, DeviceState(lat, P.data; density=true, precision=precision))
end
function _state_lattice(state, ctx)
    l = LatticeModels.lattice(state)
    LatticeModels.internal_length(state) == 1 || return context_lattice(ctx)
    try
        return device_lattice(l; ctx=ctx)
    catch e
        e isa ArgumentError || rethrow()
        return context_lattice(ctx)
    end
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
    check(ccall((:lm_solver_update, LIB), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Cdouble, Cint),
                s.handle, handle(H), dt, force), s.ctx.handle)
end
step!(s::ChebyshevGPU, st::DeviceState, _cache) =
    check(ccall((:lm_solver_step, LIB), Cint, (Ptr{Cvoid}, Ptr{Cvoid}), s.handle, st.handle), s.ctx.handle)
step!(s::ChebyshevGPU, v::DeviceVector, cache) = step!(s, v.st, cache)
evolution_cache(::ChebyshevGPU, ::Union{DeviceState,DeviceVector}) = nothing

# ---- readouts ---------------------------------------------------------------------------------
# localdensity of every row of a device state (site x internal state), summed on the device
function row_density(st::DeviceState)
    out = Vector{Float64}(undef, st.n)
    check(ccall((:lm_localdensity, LIB), Cint, (Ptr{Cvoid}, Ptr{Float64}), st.handle, out), st.lat.ctx.handle)
    return out
end
function bond_currents(H::DeviceHamiltonian, st::DeviceState)
    nb = ccall((:lm_lattice_nbonds, LIB), Int64, (Ptr{Cvoid},), H.lat.handle)
    out = Vector{Float64}(undef, nb)
    check(ccall((:lm_bond_currents, LIB), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Float64}), handle(H), st.handle, out),
          st.lat.ctx.handle)
    return out
end

# (src, dst) of every nearest-neighbour bond, 1-based, in the reference's bond order
const _BONDS = IdDict{DeviceLattice,Tuple{Vector{Int64},Vector{Int64}}}()
function lattice_bonds(lat::DeviceLattice)
    get!(_BONDS, lat) do
        nb = ccall((:lm_lattice_nbonds, LIB), Int64, (Ptr{Cvoid},), lat.handle)
        src, dst = Vector{Int64}(undef, nb), Vector{Int64}(undef, nb)
        check(ccall((:lm_lattice_bonds, LIB), Cint, (Ptr{Cvoid}, Ptr{Int64}, Ptr{Int64}), lat.handle, src, dst),
              lat.ctx.handle)
        (src, dst)
    end
end

# Reference states whose `.data` lives on the device: a density matrix (Operator) or a Ket
const DeviceOperator = QuantumOpticsBase.Operator{<:Any,<:Any,<:DeviceState}
const DeviceKet = QuantumOpticsBase.Ket{<:Any,<:DeviceVector}
device_data(op::DeviceOperator) = op.data
device_data(ket::DeviceKet) = ket.data.st

"""
    localdensity(state)

The reference's `localdensity` (src/operators/latticeutils.jl:41-45) of a device-backed `Ket`
or density-matrix `Operator`: a `LatticeValue` on the state's lattice, with the internal
states of a site summed.  The sum over the block runs on the device.
"""
function localdensity(state::Union{DeviceOperator,DeviceKet})
    l = LatticeModels.lattice(state)
    N = LatticeModels.internal_length(state)
    v = row_density(device_data(state))
    return LatticeModels.LatticeValue(l, N == 1 ? v : vec(sum(reshape(v, N, :), dims=1)))
end

LinearAlgebra.tr(st::DeviceState) = gpu_trace(st)

# DensityCurrents(H, P) (src/zoo/currents.jl:81-102) with H from GPUBuilder and a device state:
# the struct stays the reference's lazy object; its values come from one device readout of
# every bond (lm_bond_currents, J_b = 2 Im(H[i,j] P[j,i]) in the reference bond order).
const GPUDensityCurrents = DensityCurrents{<:LatticeModels.Hamiltonian{<:Any,<:Any,<:DeviceHamiltonian},
                                           <:Union{DeviceOperator,DeviceKet}}

device_bond_currents(curr::GPUDensityCurrents) = bond_currents(curr.hamiltonian.data, device_data(curr.state))

# curr[i, j]: every bond between sites i and j, taken with its direction.  Each call reads the
# bonds out of the device; materialise with `Currents(curr)` to read many pairs.
function Base.getindex(curr::GPUDensityCurrents, i::Int, j::Int)
    J = device_bond_currents(curr)
    src, dst = lattice_bonds(curr.hamiltonian.data.lat)
    v = 0.0
    for b in eachindex(J)
        src[b] == i && dst[b] == j && (v += J[b])
        src[b] == j && dst[b] == i && (v -= J[b])
    end
    return v
end

# Currents(curr) (src/currents.jl:223-237): the antisymmetric sparse matrix from one device
# readout; |J| < CURRENTS_EPS is dropped, as the reference does.  The only nonzero pairs of a
# nearest-neighbour Hamiltonian are its bonds, so Currents(curr, NearestNeighbor(1)) is the same.
function Currents(curr::GPUDensityCurrents)
    lat = LatticeModels.lattice(curr)
    J = device_bond_currents(curr)
    src, dst = lattice_bonds(curr.hamiltonian.data.lat)
    n = length(lat)
    mat = sparse(vcat(src, dst), vcat(dst, src), vcat(J, -J), n, n)  # parallel bonds add up
    Is, Js, Vs = Int[], Int[], Float64[]
    rows = rowvals(mat)
    vals = mat.nzval
    for c in 1:n, p in nzrange(mat, c)
        abs(vals[p]) < LatticeModels.CURRENTS_EPS && continue
        push!(Is, rows[p]); push!(Js, c); push!(Vs, vals[p])
    end
    return Currents(lat, sparse(Is, Js, Vs, n, n))
end
Currents(curr::GPUDensityCurrents, ::LatticeModels.NearestNeighbor{1}) = Currents(curr)

# ---- general sparse Hamiltonians: any construct_operator output (honeycomb, kagome, qwz, ...) ----
# The reference's SparseMatrixCSC goes to the device as an ELL table; update_solver! picks the
# ELL propagator, step! and the readouts are unchanged.
mutable struct GPUSparseHamiltonian <: AbstractMatrix{ComplexF64}
    ctx::Context
    handle::Ptr{Cvoid}
    n::Int
end
Base.size(H::GPUSparseHamiltonian) = (H.n, H.n)
function GPUSparseHamiltonian(A::SparseMatrixCSC{ComplexF64,Int64}; ctx=default_context())
    h = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:lm_ell_create_csc, LIB), Cint, (Ptr{Cvoid}, Int64, Ptr{Int64}, Ptr{Int64}, Ptr{ComplexF64}, Ref{Ptr{Cvoid}}),
                ctx.handle, size(A, 1), A.colptr, A.rowval, A.nzval, h), ctx.handle)
    H = GPUSparseHamiltonian(ctx, h[], size(A, 1))
    finalizer(H -> ccall((:lm_ell_destroy, LIB), Cint, (Ptr{Cvoid},), H.handle), H)
    return H
end
set_values!(H::GPUSparseHamiltonian, A::SparseMatrixCSC{ComplexF64,Int64}) =
    check(ccall((:lm_ell_set_values, LIB), Cint, (Ptr{Cvoid}, Ptr{ComplexF64}), H.handle, A.nzval), H.ctx.handle)
# An a x b HoneycombLattice in the reference's site order (unit cells (j1, j2), j2 fastest, two
# basis sites): ComplexF32 kets then step through the temporally blocked streaming kernel as an
# a x 2b brick lattice.  The library checks that every stored entry is a nearest-neighbour bond.
honeycomb_layout!(H::GPUSparseHamiltonian, a::Integer, b::Integer; periodic=(false, false)) =
    check(ccall((:lm_ell_set_layout, LIB), Cint, (Ptr{Cvoid}, Cint, Int64, Int64, Cint, Cint),
                H.handle, Cint(1), a, b, Cint(periodic[1]), Cint(periodic[2])), H.ctx.handle)
update_solver!(s::ChebyshevGPU, H::GPUSparseHamiltonian, dt, force=false) =
    check(ccall((:lm_ell_solver_update, LIB), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Cdouble, Cint), s.handle, H.handle, dt, force),
          s.ctx.handle)

# DensityCurrents(H, state)[i, j] = 2 Im(H[i,j] P[j,i]) (src/zoo/currents.jl:92-102) for every
# stored entry of A (the CSC the device table was made from), in its order; 0 on the diagonal.
function gpu_entry_currents(H::GPUSparseHamiltonian, A::SparseMatrixCSC{ComplexF64,Int64}, st)
    out = Vector{Float64}(undef, nnz(A))
    check(ccall((:lm_ell_currents, LIB), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Float64}), H.handle, st.handle, out),
          H.ctx.handle)
    return SparseMatrixCSC(size(A)..., copy(A.colptr), copy(A.rowval), out)
end

# LocalOperatorCurrents(H, state, op) (src/zoo/currents.jl:150-184) on a general Hamiltonian with
# ndof internal states per site: one device pass gives every stored entry's share, the site-pair
# value is the sum over its block (`sparse` adds the duplicates).  op === nothing: DensityCurrents.
function gpu_operator_currents(H::GPUSparseHamiltonian, A::SparseMatrixCSC{ComplexF64,Int64}, st, ndof::Integer,
                               op=nothing)
    out = Vector{Float64}(undef, nnz(A))
    opm = op === nothing ? Ptr{ComplexF64}(C_NULL) : convert(Matrix{ComplexF64}, op)
    check(ccall((:lm_ell_op_currents, LIB), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Cint, Ptr{ComplexF64}, Ptr{Float64}),
                H.handle, st.handle, ndof, opm, out), H.ctx.handle)
    return site_pair_currents(A, out, ndof)
end

# Per-entry shares (CSC order of A) -> site-pair matrix M[i, j] = curr[i, j].
function site_pair_currents(A::SparseMatrixCSC, out::AbstractVector{Float64}, ndof::Integer)
    I, J, V = Int[], Int[], Float64[]
    rows = rowvals(A)
    for c in 1:size(A, 2), p in nzrange(A, c)
        si, sj = (rows[p] - 1) ÷ ndof + 1, (c - 1) ÷ ndof + 1
        si == sj && continue
        push!(I, si); push!(J, sj); push!(V, out[p])
    end
    ns = size(A, 1) ÷ ndof
    return sparse(I, J, V, ns, ns)  # M[i, j] = curr[i, j]
end

# ---- readout ring behind TimeSequence(f, ev(times)) (src/timesequence.jl:41-43) --------------
# Readouts are computed into device ring slots and downloaded asynchronously; entries are taken
# only when their slot is about to be reused, so the evolution never waits on a readout.
mutable struct ReadoutRing
    ctx::Context
    handle::Ptr{Cvoid}
    nslots::Int
end
function ReadoutRing(len::Integer, nslots::Integer=8; ctx=default_context())
    h = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:lm_ring_create, LIB), Cint, (Ptr{Cvoid}, Cint, Int64, Ref{Ptr{Cvoid}}), ctx.handle, nslots, len, h),
          ctx.handle)
    r = ReadoutRing(ctx, h[], nslots)
    finalizer(r -> ccall((:lm_ring_destroy, LIB), Cint, (Ptr{Cvoid},), r.handle), r)
    return r
end
function push_density!(r::ReadoutRing, st::DeviceState, t)
    seq = Ref{Int64}(0)
    check(ccall((:lm_ring_push_localdensity, LIB), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Cdouble, Ref{Int64}),
                r.handle, st.handle, t, seq), r.ctx.handle)
    return seq[]
end
function push_currents!(r::ReadoutRing, H::DeviceHamiltonian, st::DeviceState, t)
    seq = Ref{Int64}(0)
    check(ccall((:lm_ring_push_currents, LIB), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Cdouble, Ref{Int64}),
                r.handle, handle(H), st.handle, t, seq), r.ctx.handle)
    return seq[]
end
function push_op_currents!(r::ReadoutRing, H::GPUSparseHamiltonian, st, ndof::Integer, t, op=nothing)
    seq = Ref{Int64}(0)
    opm = op === nothing ? Ptr{ComplexF64}(C_NULL) : convert(Matrix{ComplexF64}, op)
    check(ccall((:lm_ring_push_op_currents, LIB), Cint,
                (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Cint, Ptr{ComplexF64}, Cdouble, Ref{Int64}),
                r.handle, H.handle, st.handle, ndof, opm, t, seq), r.ctx.handle)
    return seq[]
end
function ring_take!(r::ReadoutRing, seq::Integer, len::Integer)
    out = Vector{Float64}(undef, len)
    n = Ref{Int64}(0)
    t = Ref{Cdouble}(0.0)
    check(ccall((:lm_ring_wait, LIB), Cint, (Ptr{Cvoid}, Int64, Ptr{Float64}, Ptr{Cvoid}, Ref{Int64}, Ref{Cdouble}),
                r.handle, seq, out, C_NULL, n, t), r.ctx.handle)
    return t[], resize!(out, n[])
end

"""
    gpu_timesequence(kind, ev_iter; nslots=8)

`TimeSequence(moment -> localdensity(moment.state), ev_iter)` (`kind = :density`, LatticeValue
entries) or the bond currents of `DensityCurrents(moment.H, moment.state)` (`kind =
:currents`, one value per bond in the reference bond order), read out through a `ReadoutRing`
(src/timesequence.jl:41-43).
"""
gpu_timesequence(kind::Symbol, ev_iter; nslots=8) = only(gpu_timesequences((kind,), ev_iter; nslots=nslots))

"""
    gpu_timesequences(kinds, ev_iter; nslots=8)

One `TimeSequence` per kind (`:density`, `:currents`) from a single pass over `ev_iter`: the
loop of the reference README, which reads `localdensity(P)` and `DensityCurrents(H, P)` at
every moment.  Each readout goes into its own ring; entries are collected only when their
slot is about to be reused, so the evolution never waits on a readout.
"""
function gpu_timesequences(kinds, ev_iter; nslots=8)
    rings = Any[nothing for _ in kinds]
    lens = zeros(Int, length(kinds))
    pending = [Int64[] for _ in kinds]
    ts = [Float64[] for _ in kinds]
    vals = [Any[] for _ in kinds]
    wrap = Any[identity for _ in kinds]
    collect_one!(k) = ((t, v) = ring_take!(rings[k], popfirst!(pending[k]), lens[k]); push!(ts[k], t); push!(vals[k], wrap[k](v)))
    for moment in ev_iter
        st = device_data(moment.state)
        for (k, kind) in enumerate(kinds)
            if rings[k] === nothing
                lens[k] = kind === :density ? st.n :
                          Int(ccall((:lm_lattice_nbonds, LIB), Int64, (Ptr{Cvoid},), moment.H.data.lat.handle))
                rings[k] = ReadoutRing(max(lens[k], 1), nslots; ctx=st.lat.ctx)
                if kind === :density
                    l = LatticeModels.lattice(moment.state)
                    N = LatticeModels.internal_length(moment.state)
                    wrap[k] = v -> LatticeModels.LatticeValue(l, N == 1 ? v : vec(sum(reshape(v, N, :), dims=1)))
                end
            end
            length(pending[k]) == nslots && collect_one!(k)
            push!(pending[k], kind === :density ? push_density!(rings[k], st, moment.t) :
                                                  push_currents!(rings[k], moment.H.data::DeviceHamiltonian, st, moment.t))
        end
    end
    for k in eachindex(kinds)
        while !isempty(pending[k])
            collect_one!(k)
        end
    end
    return [LatticeModels.TimeSequence(ts[k], vals[k]) for k in eachindex(kinds)]
end

"""
    gpu_operator_timesequence(H, A, ev_iter, ndof; op=nothing, nslots=8)

`TimeSequence(moment -> LocalOperatorCurrents(H, moment.state, op), ev_iter)` for a general
(sparse) Hamiltonian with ndof internal states per site (src/zoo/currents.jl:150-184); `op ===
nothing` gives `DensityCurrents`.  The per-entry shares go through a `ReadoutRing`; each is
summed into site pairs on the host once its slot is taken.
"""
function gpu_operator_timesequence(H::GPUSparseHamiltonian, A::SparseMatrixCSC{ComplexF64,Int64}, ev_iter,
                                   ndof::Integer; op=nothing, nslots=8)
    ring = ReadoutRing(max(nnz(A), 1), nslots; ctx=H.ctx)
    pending = Int64[]
    ts = Float64[]
    vals = Any[]
    for moment in ev_iter
        if length(pending) == nslots
            t, v = ring_take!(ring, popfirst!(pending), nnz(A))
            push!(ts, t); push!(vals, site_pair_currents(A, v, ndof))
        end
        push!(pending, push_op_currents!(ring, H, device_data(moment.state), ndof, moment.t, op))
    end
    for seq in pending
        t, v = ring_take!(ring, seq, nnz(A))
        push!(ts, t); push!(vals, site_pair_currents(A, v, ndof))
    end
    return LatticeModels.TimeSequence(ts, vals)
end

# ---- batches of uneven lattices (lm_batch_*) ---------------------------------------------------
mutable struct GPUBatch
    ctx::Context
    handle::Ptr{Cvoid}
    members::Vector{Any}  # keeps the Hamiltonians and states alive
end
function GPUBatch(kind::Cint, precision::Cint; tol=precision == LM_C32 ? 1e-9 : 1e-12, ctx=default_context())
    h = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:lm_batch_create, LIB), Cint, (Ptr{Cvoid}, Cint, Cint, Cdouble, Ref{Ptr{Cvoid}}),
                ctx.handle, kind, precision, tol, h), ctx.handle)
    b = GPUBatch(ctx, h[], Any[])
    finalizer(b -> ccall((:lm_batch_destroy, LIB), Cint, (Ptr{Cvoid},), b.handle), b)
    return b
end
function Base.push!(b::GPUBatch, H::DeviceHamiltonian, st::DeviceState)
    idx = Ref{Cint}(0)
    slot = private_slot(H)
    check(ccall((:lm_batch_add, LIB), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ref{Cint}), b.handle, slot.handle,
                st.handle, idx), b.ctx.handle)
    push!(b.members, (slot, st))
    return b
end
update!(b::GPUBatch, dt) = check(ccall((:lm_batch_update, LIB), Cint, (Ptr{Cvoid}, Cdouble), b.handle, dt), b.ctx.handle)
step!(b::GPUBatch) = check(ccall((:lm_batch_step, LIB), Cint, (Ptr{Cvoid},), b.handle), b.ctx.handle)
function tune!(b::GPUBatch; steps=2)
    ms = Vector{Float64}(undef, 4)
    best = Ref{Cint}(0)
    check(ccall((:lm_batch_tune, LIB), Cint, (Ptr{Cvoid}, Cint, Ptr{Float64}, Ref{Cint}), b.handle, steps, ms, best),
          b.ctx.handle)
    return best[], ms
end

# ---- adjoint: ChainRulesCore rrule of a density loss (lm_adjoint_*) -----------------------------
# loss(V, B) = sum_i (localdensity_i(T) - target_i)^2 after `nsteps` steps of dt under
# gpu_tightbinding(l, V; field=PointFlux(B[j], point)), B piecewise constant over `spi` steps.
# The forward pass keeps a checkpoint every `every` steps; the pullback recomputes each segment,
# runs lm_adjoint_step per step and propagates the co-state with a solver at -dt.  This mirrors
# DensityLossAdjoint of the Python host (latticemodels.jl_gb300/lmgpu/adjoint.py) call for call.
struct DensityLossProblem
    lat::DeviceLattice
    psi0::Matrix{ComplexF64}
    target::Vector{Float64}
    dt::Float64
    nsteps::Int
    spi::Int
    point::NTuple{2,Float64}
    precision::Cint
    every::Int
    bounds::NTuple{2,Float64}
end

"""
    loss_and_gradients(p, V, B) -> (loss, dL/dV, dL/dB)

The density loss after the forward pass and its gradients from the hand-written adjoint: the
forward pass keeps a checkpoint every `p.every` steps, the backward pass recomputes each
segment, runs lm_adjoint_step per step and propagates the co-state with a solver at -dt.
"""
function loss_and_gradients(p::DensityLossProblem, V::Vector{Float64}, B::Vector{Float64})
    ctx = p.lat.ctx
    tol = p.precision == LM_C32 ? 1e-9 : 1e-12
    fwd, bwd = ChebyshevGPU(; tol=tol, ctx=ctx), ChebyshevGPU(; tol=tol, ctx=ctx)
    for s in (fwd, bwd)
        check(ccall((:lm_solver_set_bounds, LIB), Cint, (Ptr{Cvoid}, Cdouble, Cdouble), s.handle, p.bounds...),
              ctx.handle)
    end
    comps = [(LM_FIELD_POINTFLUX_AXIAL, p.point...)]
    Vd = copy(V)   # one on-site array for every step: it is uploaded once
    ham(amp) = DeviceHamiltonian(p.lat, 1.0, comps, [amp], Vd, true)
    n, m = size(p.psi0)
    adj = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:lm_adjoint_create, LIB), Cint, (Ptr{Cvoid}, Int64, Int64, Cint, Cint, Ref{Ptr{Cvoid}}),
                ctx.handle, n, m, p.precision, length(B), adj), ctx.handle)
    try
        stepwith!(s, amp, dt, st) = (update_solver!(s, ham(amp), dt); step!(s, st, nothing))
        psi = DeviceState(p.lat, p.psi0; precision=p.precision)
        cps = [copy(psi)]
        for k in 1:p.nsteps
            stepwith!(fwd, B[(k - 1) ÷ p.spi + 1], p.dt, psi)
            k % p.every == 0 && k < p.nsteps && push!(cps, copy(psi))
        end
        lam = DeviceState(p.lat, zeros(ComplexF64, n, m); precision=p.precision)
        loss = Ref{Cdouble}(0.0)
        check(ccall((:lm_adjoint_seed, LIB), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Float64}, Ptr{Cvoid}, Ref{Cdouble}),
                    adj[], psi.handle, p.target, lam.handle, loss), ctx.handle)
        check(ccall((:lm_adjoint_reset, LIB), Cint, (Ptr{Cvoid},), adj[]), ctx.handle)
        for c in length(cps):-1:1
            n0 = (c - 1) * p.every
            n1 = min(p.nsteps, n0 + p.every)
            seg = [copy(cps[c])]
            for k in n0+1:n1-1
                nxt = copy(seg[end])
                stepwith!(fwd, B[(k - 1) ÷ p.spi + 1], p.dt, nxt)
                push!(seg, nxt)
            end
            for k in n1:-1:n0+1
                j = (k - 1) ÷ p.spi + 1
                Hj = ham(B[j])
                update_solver!(fwd, Hj, p.dt)
                check(ccall((:lm_adjoint_step, LIB), Cint,
                            (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Cint, Cint, Ptr{Cvoid}, Ptr{Cvoid}),
                            adj[], fwd.handle, handle(Hj), 0, j - 1, seg[k - n0].handle, lam.handle), ctx.handle)
                stepwith!(bwd, B[j], -p.dt, lam)
            end
        end
        gV = Vector{Float64}(undef, n)
        gB = Vector{Float64}(undef, length(B))
        check(ccall((:lm_adjoint_gradients, LIB), Cint, (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}), adj[], gV, gB),
              ctx.handle)
        return loss[], gV, gB
    finally
        ccall((:lm_adjoint_destroy, LIB), Cint, (Ptr{Cvoid},), adj[])
    end
end

# The loss alone; its ChainRulesCore rrule (ext/LatticeModelsGB300ChainRulesCoreExt.jl, a
# package extension loaded with ChainRulesCore) returns the adjoint gradients.
density_loss(V, B, p::DensityLossProblem) = loss_and_gradients(p, Vector{Float64}(V), Vector{Float64}(B))[1]

# ---- context options, state utilities -----------------------------------------------------------
const LM_OPT_FUSED = Cint(1)   # 0: one launch per Chebyshev order for ComplexF32 states
const LM_OPT_STREAM = Cint(2)  # 0: the region form of the fused step instead of the x-streaming form
const LM_OPT_KPM = Cint(3)     # 0: FP64 KPM and Fermi-operator recurrences instead of double-float
const LM_OPT_RESIDENT = Cint(4)  # 0: a ComplexF32 batch's lattices in the region form instead of the lattice-resident form

gpu_synchronize(ctx::Context=default_context()) =
    check(ccall((:lm_ctx_synchronize, LIB), Cint, (Ptr{Cvoid},), ctx.handle), ctx.handle)
set_option!(ctx::Context, option::Cint, value::Integer) =
    check(ccall((:lm_ctx_set_option, LIB), Cint, (Ptr{Cvoid}, Cint, Cint), ctx.handle, option, value), ctx.handle)

# Ensemble weights: P = sum_k w_k |psi_k><psi_k| for the readouts (nothing: all ones).
function set_weights!(st::DeviceState, w)
    wv = w === nothing ? Ptr{Float64}(C_NULL) : Vector{Float64}(w)
    check(ccall((:lm_state_set_weights, LIB), Cint, (Ptr{Cvoid}, Ptr{Float64}), st.handle, wv), st.lat.ctx.handle)
    return st
end
function gpu_trace(st::DeviceState)
    out = Ref{Cdouble}(0.0)
    check(ccall((:lm_trace, LIB), Cint, (Ptr{Cvoid}, Ref{Cdouble}), st.handle, out), st.lat.ctx.handle)
    return out[]
end
function gpu_norms(st::DeviceState)
    out = Vector{Float64}(undef, st.m)
    check(ccall((:lm_state_norms, LIB), Cint, (Ptr{Cvoid}, Ptr{Float64}), st.handle, out), st.lat.ctx.handle)
    return out
end
gpu_renormalize!(st::DeviceState, target::AbstractVector{<:Real}) =
    check(ccall((:lm_state_renormalize, LIB), Cint, (Ptr{Cvoid}, Ptr{Float64}), st.handle, Vector{Float64}(target)),
          st.lat.ctx.handle)
# Compensated ComplexF32 kets: keep each amplitude's rounding residual so that long FP32 runs
# do not accumulate the state's rounding (states the x-streaming step takes)
gpu_compensate!(st::DeviceState, enable::Bool=true) =
    check(ccall((:lm_state_set_compensation, LIB), Cint, (Ptr{Cvoid}, Cint), st.handle, Cint(enable)),
          st.lat.ctx.handle)
# (pointer, leading dimension) of the device block, e.g. for unsafe_wrap(CuArray, ...); it
# changes when a step swaps buffers
function device_pointer(st::DeviceState)
    p = Ref{Ptr{Cvoid}}(C_NULL)
    ld = Ref{Int64}(0)
    check(ccall((:lm_state_device_ptr, LIB), Cint, (Ptr{Cvoid}, Ref{Ptr{Cvoid}}, Ref{Int64}), st.handle, p, ld),
          st.lat.ctx.handle)
    return p[], ld[]
end
# (K, a, b): Chebyshev order and the interval [b - a, b + a] of the last update_solver!
function solver_order(s::ChebyshevGPU)
    K = Ref{Cint}(0)
    a = Ref{Cdouble}(0.0)
    b = Ref{Cdouble}(0.0)
    check(ccall((:lm_solver_order, LIB), Cint, (Ptr{Cvoid}, Ref{Cint}, Ref{Cdouble}, Ref{Cdouble}), s.handle, K, a, b),
          s.ctx.handle)
    return Int(K[]), a[], b[]
end

# ---- spectral bounds, KPM and the Fermi operator (no eigensystem) --------------------------------
# :gershgorin always encloses the spectrum; :lanczos is tighter (FP64 Lanczos, the Ritz values
# padded by their residuals and 1 % of the width, clipped to Gershgorin).
function spectral_bounds(H::DeviceHamiltonian; method=:gershgorin, iters=64, seed=0x5eed)
    lo = Ref{Cdouble}(0.0)
    hi = Ref{Cdouble}(0.0)
    ctx = H.lat.ctx.handle
    if method === :lanczos
        check(ccall((:lm_ham_lanczos_bounds, LIB), Cint, (Ptr{Cvoid}, Cint, Culonglong, Ref{Cdouble}, Ref{Cdouble}),
                    handle(H), iters, seed, lo, hi), ctx)
    else
        check(ccall((:lm_ham_bounds, LIB), Cint, (Ptr{Cvoid}, Ref{Cdouble}, Ref{Cdouble}), handle(H), lo, hi), ctx)
    end
    return lo[], hi[]
end
function padded_bounds(H::DeviceHamiltonian; method=:gershgorin)
    lo, hi = spectral_bounds(H; method=method)
    pad = 1e-3 * (hi - lo)
    return lo - pad, hi + pad
end

"""
    kpm_moments(H, nmom; vecs=nothing, per_column=false, bounds=padded_bounds(H))

KPM moments mu_n = sum_v <v|T_n(H~)|v>, n < nmom, in FP64, on the interval `bounds`
(H~ = (H - b)/a).  `vecs`: a ComplexF64 `DeviceState` of starting vectors (stochastic
trace), or `nothing` for the N unit vectors (exact trace).  `per_column=true` keeps one
column of moments per vector (with unit vectors: the local moments of every site, the LDOS).
The density of states follows from the moments without an eigensystem (the reference
computes `dos` from an Eigensystem, src/greenfunction.jl:306).
"""
function kpm_moments(H::DeviceHamiltonian, nmom::Integer; vecs=nothing, per_column=false, bounds=padded_bounds(H))
    ncol = per_column ? (vecs === nothing ? size(H, 1) : vecs.m) : 1
    out = Vector{Float64}(undef, nmom * ncol)
    vh = vecs === nothing ? C_NULL : vecs.handle
    check(ccall((:lm_kpm_moments, LIB), Cint, (Ptr{Cvoid}, Cdouble, Cdouble, Cint, Ptr{Cvoid}, Cint, Ptr{Float64}),
                handle(H), bounds[1], bounds[2], nmom, vh, per_column, out), H.lat.ctx.handle)
    return per_column ? reshape(out, nmom, ncol) : out
end

"""
    chebyshev_coefficients(f, (emin, emax); tol=1e-13)

Real Chebyshev coefficients c_n of x -> f(a x + b) on [-1, 1], with [b - a, b + a] =
(emin, emax), truncated where the tail sum_{n >= K} |c_n| is below `tol`.  They come from the
Chebyshev-Gauss nodes (a type-II DCT, summed directly); the node count doubles until the
series has converged within the first quarter of the coefficients.
"""
function chebyshev_coefficients(f, bounds; tol=1e-13, max_nodes=1 << 16)
    emin, emax = bounds
    a, b = (emax - emin) / 2, (emax + emin) / 2
    nodes = 4096
    while true
        theta = [pi * (k + 0.5) / nodes for k in 0:nodes-1]
        fx = [f(a * cos(t) + b) for t in theta]
        nc = nodes ÷ 4 + 1
        c = [2 / nodes * sum(fx[k] * cos(n * theta[k]) for k in 1:nodes) for n in 0:nc-1]
        c[1] /= 2
        tail = reverse(cumsum(reverse(abs.(c))))
        K = findfirst(<=(tol), tail)
        K !== nothing && return c[1:max(K - 1, 1)]
        nodes >= max_nodes && throw(ArgumentError("the Chebyshev series of f does not converge on the spectral interval"))
        nodes *= 2
    end
end

"""
    gpu_densitymatrix(H; mu, T, precision=LM_C64, tol=1e-13, bounds=padded_bounds(H))

`densitymatrix(H; mu, T)` for T > 0 (src/spectrum.jl:252-257) without an eigensystem: the
Chebyshev series of the FermiDirac occupation f(E) = 1 / (exp((E - mu)/T) + 1)
(src/spectrum.jl:230-232) applied to the identity on the device.  At T = 0 the occupation is a
step and its series does not converge; `densitymatrix` takes the device eigensystem there.
"""
function gpu_densitymatrix(H::DeviceHamiltonian; mu, T, precision=LM_C64, tol=1e-13, bounds=padded_bounds(H))
    T > 0 || throw(ArgumentError("the Chebyshev Fermi operator needs T > 0"))
    c = chebyshev_coefficients(E -> (1 - tanh((E - mu) / (2T))) / 2, bounds; tol=tol)
    n = size(H, 1)
    ctx = H.lat.ctx.handle
    h = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:lm_state_create, LIB), Cint, (Ptr{Cvoid}, Int64, Int64, Cint, Cint, Ref{Ptr{Cvoid}}),
                ctx, n, n, LM_DENSITY, precision, h), ctx)
    out = DeviceState(H.lat, h[], n, n, LM_DENSITY, precision)
    finalizer(s -> ccall((:lm_state_destroy, LIB), Cint, (Ptr{Cvoid},), s.handle), out)
    check(ccall((:lm_cheb_apply, LIB), Cint, (Ptr{Cvoid}, Cdouble, Cdouble, Ptr{Float64}, Cint, Ptr{Cvoid}, Ptr{Cvoid}),
                handle(H), bounds[1], bounds[2], c, length(c), C_NULL, out.handle), ctx)
    return out
end

# ---- eigensystem: diagonalize / densitymatrix at T = 0 (src/spectrum.jl:48-55, :226-257) -----
"""
    GPUEigensystem(H)

The FP64 eigensystem of a device Hamiltonian on the library's own kernels (lm_eigsys_*):
`values` in ascending order, eigenvectors and weighted projectors on demand.
"""
mutable struct GPUEigensystem
    ctx::Context
    handle::Ptr{Cvoid}
    lat::DeviceLattice
    values::Vector{Float64}
end
function GPUEigensystem(H::DeviceHamiltonian)
    h = Ref{Ptr{Cvoid}}(C_NULL)
    ctx = H.lat.ctx
    check(ccall((:lm_eigsys_create, LIB), Cint, (Ptr{Cvoid}, Ref{Ptr{Cvoid}}), handle(H), h), ctx.handle)
    return _eigsys(ctx, h[], H.lat)
end
function GPUEigensystem(H::GPUSparseHamiltonian)
    h = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:lm_eigsys_create_ell, LIB), Cint, (Ptr{Cvoid}, Ref{Ptr{Cvoid}}), H.handle, h), H.ctx.handle)
    return _eigsys(H.ctx, h[], context_lattice(H.ctx))
end
function _eigsys(ctx::Context, h::Ptr{Cvoid}, lat::DeviceLattice)
    n = Ref{Int64}(0)
    check(ccall((:lm_eigsys_size, LIB), Cint, (Ptr{Cvoid}, Ref{Int64}), h, n), ctx.handle)
    w = Vector{Float64}(undef, n[])
    check(ccall((:lm_eigsys_values, LIB), Cint, (Ptr{Cvoid}, Ptr{Float64}), h, w), ctx.handle)
    e = GPUEigensystem(ctx, h, lat, w)
    finalizer(e -> ccall((:lm_eigsys_destroy, LIB), Cint, (Ptr{Cvoid},), e.handle), e)
    return e
end
# eigenvectors first .. first + m - 1 as an n x m device ket block
function eigenvectors(e::GPUEigensystem, first::Integer=1, m::Integer=length(e.values) - first + 1; precision=LM_C64)
    n = length(e.values)
    h = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:lm_state_create, LIB), Cint, (Ptr{Cvoid}, Int64, Int64, Cint, Cint, Ref{Ptr{Cvoid}}),
                e.ctx.handle, n, m, LM_KETS, precision, h), e.ctx.handle)
    out = DeviceState(e.lat, h[], n, m, LM_KETS, precision)
    finalizer(s -> ccall((:lm_state_destroy, LIB), Cint, (Ptr{Cvoid},), s.handle), out)
    check(ccall((:lm_eigsys_vectors, LIB), Cint, (Ptr{Cvoid}, Int64, Ptr{Cvoid}), e.handle, first - 1, out.handle),
          e.ctx.handle)
    return out
end
# sum_k w_k v_k v_k^H as an n x n device density matrix
function projector(e::GPUEigensystem, w::AbstractVector{<:Real}; precision=LM_C64)
    n = length(e.values)
    length(w) == n || throw(DimensionMismatch("one weight per eigenvalue"))
    h = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:lm_state_create, LIB), Cint, (Ptr{Cvoid}, Int64, Int64, Cint, Cint, Ref{Ptr{Cvoid}}),
                e.ctx.handle, n, n, LM_DENSITY, precision, h), e.ctx.handle)
    out = DeviceState(e.lat, h[], n, n, LM_DENSITY, precision)
    finalizer(s -> ccall((:lm_state_destroy, LIB), Cint, (Ptr{Cvoid},), s.handle), out)
    check(ccall((:lm_eigsys_projector, LIB), Cint, (Ptr{Cvoid}, Ptr{Float64}, Ptr{Cvoid}), e.handle,
                Vector{Float64}(w), out.handle), e.ctx.handle)
    return out
end

# "E == mu" at T = 0 (src/spectrum.jl:230-232) is |E - mu| <= 1e-12 max(1, |E|max): a level
# that is exactly degenerate at mu is occupied as a whole, not split by rounding.
degenerate_tol(w) = 1e-12 * max(1.0, maximum(abs, w; init=0.0))

"""
    densitymatrix(H; mu, T=0, precision=LM_C64)

The reference's `densitymatrix` (src/spectrum.jl:226-257, :317-333) for a Hamiltonian built
with `GPUBuilder`: an `Operator` whose `.data` is a `DeviceState`.  T > 0: the Chebyshev series
of the FermiDirac occupation on the device (`gpu_densitymatrix`); T = 0: the device eigensystem
with the occupied levels E <= mu (E == mu occupied, as the reference's densfun does).
"""
function densitymatrix(ham::LatticeModels.Hamiltonian{<:Any,<:Any,<:DeviceHamiltonian}; mu=nothing, μ=mu, T=0,
                       precision=LM_C64)
    mu = something(μ, 0.0)
    H = ham.data
    st = if T > 0
        gpu_densitymatrix(H; mu=mu, T=T, precision=precision)
    else
        e = GPUEigensystem(H)
        tol = degenerate_tol(e.values)
        projector(e, [E - mu <= tol ? 1.0 : 0.0 for E in e.values]; precision=precision)
    end
    return QuantumOpticsBase.Operator(QuantumOpticsBase.basis(ham), st)
end

export GPUBuilder, ChebyshevGPU, DeviceLattice, DeviceState, DeviceVector, DeviceHamiltonian, to_device,
       gpu_tightbinding, bond_currents, lattice_bonds, ReadoutRing, gpu_timesequence, gpu_timesequences,
       loss_and_gradients, GPUEigensystem, eigenvectors, projector, GPUBatch, DensityLossProblem, density_loss, GPUSparseHamiltonian, set_values!, gpu_operator_currents,
       gpu_operator_timesequence, gpu_synchronize, set_option!, set_weights!, gpu_trace, gpu_norms, gpu_renormalize!, gpu_compensate!, honeycomb_layout!,
       device_pointer, solver_order, spectral_bounds, padded_bounds, kpm_moments, chebyshev_coefficients,
       gpu_densitymatrix, gpu_entry_currents, LM_OPT_FUSED, LM_OPT_STREAM, LM_OPT_KPM, LM_OPT_RESIDENT

end # module
