# LatticeModelsGB300 — Julia glue for the GB300 evolution backend (liblmgpu.so).
#
# Adds `ChebyshevGPU <: LatticeModels.EvolutionSolver` and a lazy device Hamiltonian so that
#     Evolution(ChebyshevGPU(tol=1e-12), t -> gpu_tightbinding(l; field=PointFlux(B(t), p)), P0)
# runs the reference's own `Evolution` driver (src/evolution.jl:183-298) on the GPU.
# Every call goes through the C ABI declared in include/lmgpu.h.
module LatticeModelsGB300

using LatticeModels
import LatticeModels: EvolutionSolver, update_solver!, step!, evolution_cache, localdensity
using SparseArrays: SparseMatrixCSC, nnz, nzrange, rowvals, sparse

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
                r.handle, H.handle, st.handle, t, seq), r.ctx.handle)
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

`TimeSequence(moment -> localdensity(moment.state), ev_iter)` (`kind = :density`) or the bond
currents of `DensityCurrents(moment.H, moment.state)` (`kind = :currents`), read out through a
`ReadoutRing`.
"""
function gpu_timesequence(kind::Symbol, ev_iter; nslots=8)
    ring = nothing
    len = 0
    pending = Int64[]
    ts = Float64[]
    vals = Vector{Vector{Float64}}()
    for moment in ev_iter
        st = moment.state.data::DeviceState
        if ring === nothing
            len = kind === :density ? st.n :
                  Int(ccall((:lm_lattice_nbonds, LIB), Int64, (Ptr{Cvoid},), st.lat.handle))
            ring = ReadoutRing(max(len, 1), nslots; ctx=st.lat.ctx)
        end
        if length(pending) == nslots
            t, v = ring_take!(ring, popfirst!(pending), len)
            push!(ts, t); push!(vals, v)
        end
        push!(pending, kind === :density ? push_density!(ring, st, moment.t) :
                                           push_currents!(ring, moment.H.data::DeviceHamiltonian, st, moment.t))
    end
    for seq in pending
        t, v = ring_take!(ring, seq, len)
        push!(ts, t); push!(vals, v)
    end
    return LatticeModels.TimeSequence(ts, vals)
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
        push!(pending, push_op_currents!(ring, H, moment.state.data, ndof, moment.t, op))
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
    check(ccall((:lm_batch_add, LIB), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ref{Cint}), b.handle, H.handle,
                st.handle, idx), b.ctx.handle)
    push!(b.members, (H, st))
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

function _loss_and_grad(p::DensityLossProblem, V::Vector{Float64}, B::Vector{Float64})
    ctx = p.lat.ctx
    tol = p.precision == LM_C32 ? 1e-9 : 1e-12
    fwd, bwd = ChebyshevGPU(; tol=tol, ctx=ctx), ChebyshevGPU(; tol=tol, ctx=ctx)
    for s in (fwd, bwd)
        check(ccall((:lm_solver_set_bounds, LIB), Cint, (Ptr{Cvoid}, Cdouble, Cdouble), s.handle, p.bounds...),
              ctx.handle)
    end
    H = gpu_tightbinding(p.lat, V; field=PointFlux(B[1], p.point))
    n, m = size(p.psi0)
    adj = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:lm_adjoint_create, LIB), Cint, (Ptr{Cvoid}, Int64, Int64, Cint, Cint, Ref{Ptr{Cvoid}}),
                ctx.handle, n, m, p.precision, length(B), adj), ctx.handle)
    try
        stepwith!(s, amp, dt, st) = (H.amplitudes[1] = amp; update_solver!(s, H, dt); step!(s, st, nothing))
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
                H.amplitudes[1] = B[j]
                update_solver!(fwd, H, p.dt)
                check(ccall((:lm_adjoint_step, LIB), Cint,
                            (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Cint, Cint, Ptr{Cvoid}, Ptr{Cvoid}),
                            adj[], fwd.handle, H.handle, 0, j - 1, seg[k - n0].handle, lam.handle), ctx.handle)
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

density_loss(V, B, p::DensityLossProblem) = _loss_and_grad(p, Vector{Float64}(V), Vector{Float64}(B))[1]

# ChainRulesCore is a weak dependency: this block is an extension (ext/ChainRulesCoreExt.jl in a
# package layout) so LatticeModels does not depend on it.
import ChainRulesCore
function ChainRulesCore.rrule(::typeof(density_loss), V, B, p::DensityLossProblem)
    loss, gV, gB = _loss_and_grad(p, Vector{Float64}(V), Vector{Float64}(B))
    pullback(dl) = (ChainRulesCore.NoTangent(), dl .* gV, dl .* gB, ChainRulesCore.NoTangent())
    return loss, pullback
end

# ---- context options, state utilities -----------------------------------------------------------
const LM_OPT_FUSED = Cint(1)   # 0: one launch per Chebyshev order for ComplexF32 states
const LM_OPT_STREAM = Cint(2)  # 0: the region form of the fused step instead of the x-streaming form
const LM_OPT_KPM = Cint(3)     # 0: FP64 KPM and Fermi-operator recurrences instead of double-float

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
                    H.handle, iters, seed, lo, hi), ctx)
    else
        check(ccall((:lm_ham_bounds, LIB), Cint, (Ptr{Cvoid}, Ref{Cdouble}, Ref{Cdouble}), H.handle, lo, hi), ctx)
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
                H.handle, bounds[1], bounds[2], nmom, vh, per_column, out), H.lat.ctx.handle)
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
step and its series does not converge; that case keeps the eigensystem route.
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
                H.handle, bounds[1], bounds[2], c, length(c), C_NULL, out.handle), ctx)
    return out
end

export ChebyshevGPU, DeviceLattice, DeviceState, gpu_tightbinding, bond_currents, ReadoutRing,
       gpu_timesequence, GPUBatch, DensityLossProblem, density_loss, GPUSparseHamiltonian, set_values!, gpu_operator_currents,
       gpu_operator_timesequence, gpu_synchronize, set_option!, set_weights!, gpu_trace, gpu_norms, gpu_renormalize!,
       device_pointer, solver_order, spectral_bounds, padded_bounds, kpm_moments, chebyshev_coefficients,
       gpu_densitymatrix, gpu_entry_currents, LM_OPT_FUSED, LM_OPT_STREAM, LM_OPT_KPM

end # module
