"""
    DeoGB300

Julia-side shim that routes DiffEqOperators.jl's stencil applies on `CuArray`s
to libdeo (include/deo.h) through `ccall`.  It adds methods for `mul!` and `*`
on the reference's own types when the array is a `CuArray{Float64}` or
`CuArray{Float32}`; CPU arrays keep the reference's methods.

The operator's tables are passed as they are stored in the reference's
`DerivativeOperator` (deo_operator_from_tables), so the device applies use
exactly the reference's coefficients.

Not exercised in this repository's test-suite: no Julia toolchain is available
where it was built.  The same C ABI is exercised from Python (deo/_lib.py).
"""
module DeoGB300

using LinearAlgebra
using Libdl
using CUDA
using DiffEqOperators
using DiffEqOperators: DerivativeOperator, GhostDerivativeOperator, DiffEqOperatorCombination,
                       AffineBC, PeriodicBC, MultiDimDirectionalBC, ComposedMultiDimBC

const libdeo = get(ENV, "DEO_LIB", joinpath(@__DIR__, "..", "libdeo.so"))
const DEO_MAX_BC = 16

# ---- C structs (layouts match include/deo.h) --------------------------------
struct DeoOperatorDesc
    derivative_order::Cint
    approximation_order::Cint
    len::Cint
    stencil_length::Cint
    boundary_stencil_length::Cint
    boundary_point_count::Cint
    offside::Cint
    winding::Cint
    uniform::Cint
    coeff_func_sign::Cint
    n_stencil_rows::Cint
    n_low_rows::Cint
    n_high_rows::Cint
    stencil_coefs::Ptr{Cdouble}
    low_boundary_coefs::Ptr{Cdouble}
    high_boundary_coefs::Ptr{Cdouble}
    coefficients::Ptr{Cdouble}
end

struct DeoBC
    kind::Cint
    m_l::Cint
    m_r::Cint
    a_l::NTuple{DEO_MAX_BC,Cdouble}
    a_r::NTuple{DEO_MAX_BC,Cdouble}
    b_l::Cdouble
    b_r::Cdouble
end

struct DeoTerm
    op::Ptr{Cvoid}
    axis::Cint
    bc::Ptr{DeoBC}
    coeff_field::Ptr{Cvoid}
    path::Cint
    line_bcs::Ptr{DeoBC}  # C_NULL, or one BC per line (MultiDimBC{dim}(BCs::Array))
end

# ---- errors: deo_status -> the reference's exception types ------------------
function check(status::Cint)
    status == 0 && return nothing
    msg = unsafe_string(ccall((:deo_last_error, libdeo), Cstring, ()))
    status == 1 && throw(DimensionMismatch(msg))          # DEO_ERR_BAD_SHAPE
    status == 2 && throw(ArgumentError(msg))              # DEO_ERR_BAD_ARG
    error("libdeo status $status: $msg")
end

# ---- operators: flatten a DerivativeOperator's fields ------------------------
_flat(v::AbstractVector{<:AbstractVector}) = Float64.(reduce(vcat, collect.(v); init = Float64[]))
_flat(v::AbstractVector{<:Real}) = Float64.(collect(v))
function _flat(m::AbstractMatrix)   # non-uniform UpwindDifference: 2 x n SMatrix of SVectors
    Float64.(vcat(_flat(vec(m[1, :])), _flat(vec(m[2, :]))))
end

function deo_operator(L::DerivativeOperator{T}) where {T}
    wind = DiffEqOperators.use_winding(L)
    uniform = L.dx isa Number
    st, lo, hi = _flat(L.stencil_coefs), _flat(L.low_boundary_coefs), _flat(L.high_boundary_coefs)
    halves = (wind && !uniform) ? 2 : 1
    coeff = L.coefficients === nothing ? ones(Float64, L.len) :
            L.coefficients isa Number ? fill(Float64(L.coefficients), L.len) : Float64.(L.coefficients)
    cfs = L.coeff_func isa Number ? (L.coeff_func >= 0 ? 1 : -1) : 0
    d = DeoOperatorDesc(L.derivative_order, L.approximation_order, L.len, L.stencil_length,
                        L.boundary_stencil_length, L.boundary_point_count, L.offside, wind, uniform, cfs,
                        div(length(st), halves * L.stencil_length),
                        div(length(lo), max(1, halves * L.boundary_stencil_length)),
                        div(length(hi), max(1, halves * L.boundary_stencil_length)),
                        pointer(st), pointer(lo), pointer(hi), pointer(coeff))
    h = Ref{Ptr{Cvoid}}(C_NULL)
    GC.@preserve st lo hi coeff check(ccall((:deo_operator_from_tables, libdeo), Cint,
                                            (Ref{DeoOperatorDesc}, Ref{Ptr{Cvoid}}), d, h))
    return h[]
end

_pad(v) = ntuple(i -> i <= length(v) ? Float64(v[i]) : 0.0, DEO_MAX_BC)
deo_bc(Q::AffineBC) = DeoBC(0, length(Q.a_l), length(Q.a_r), _pad(Q.a_l), _pad(Q.a_r), Q.b_l, Q.b_r)
deo_bc(::PeriodicBC) = DeoBC(1, 0, 0, _pad(()), _pad(()), 0.0, 0.0)
_axis(::DerivativeOperator{T, N}) where {T, N} = N

# BCs acting on axis `ax` of an N-D array: the array of per-line BCs
# (multi_dim_bc_operators.jl:54-61; MultiDimBC{dim}(BC, s) fills it with one
# BC, MultiDimBC{dim}(BCs::Array) gives one per line), or an atomic BC
_line_bcs(Q::Union{AffineBC, PeriodicBC}, ax) = nothing
_line_bcs(Q::MultiDimDirectionalBC, ax) = Q.BCs
_line_bcs(Q::ComposedMultiDimBC, ax) = Q.BCs[ax]
_bc_for(Q::Union{AffineBC, PeriodicBC}, ax) = Q
_bc_for(Q::Union{MultiDimDirectionalBC, ComposedMultiDimBC}, ax) = first(_line_bcs(Q, ax))
# libdeo's per-line table (column-major over the other axes, the array's own
# order); C_NULL-equivalent `nothing` when every line has the same BC
function _deo_line_bcs(Q, ax)
    B = _line_bcs(Q, ax)
    (B === nothing || all(b -> b === first(B) || deo_bc(b) == deo_bc(first(B)), B)) && return nothing
    return DeoBC[deo_bc(b) for b in vec(B)]
end

_ghosts(A::GhostDerivativeOperator) = (A,)
_ghosts(A::DiffEqOperatorCombination) = Tuple(op for op in A.ops)

# Device plans hold the operators' coefficients.  update_coefficients!
# (abstract_operator_functions.jl:190-194) lets a coeff_func rewrite
# L.coefficients in place, so every cache key below carries the coefficient
# values: a changed vector builds a new plan instead of reusing a stale one.
_coeff_key(L::DerivativeOperator) = hash(L.coefficients)
_coeff_key(A::GhostDerivativeOperator) = _coeff_key(A.L)
_coeff_key(A::DiffEqOperatorCombination) = hash(map(_coeff_key, A.ops))

# The plan of `cache` for (shape key, coefficient key); plans built for earlier
# coefficient values of the same shape are destroyed (`destroy`, a libdeo
# *_destroy symbol) so that a coeff_func updated every step does not pile up plans.
function _cached!(make, cache::Dict, shape_key, ckey, destroy::Symbol)
    k = (shape_key, ckey)
    haskey(cache, k) && return cache[k]
    for kk in collect(keys(cache))
        if kk[1] == shape_key
            h = pop!(cache, kk)
            ccall(Libdl.dlsym(Libdl.dlopen(libdeo), destroy), Cvoid, (Ptr{Cvoid},), h)
        end
    end
    return cache[k] = make()
end

# ---- plans (cached per operator object, size, element type and coefficients) -
const PLANS = IdDict{Any, Dict{Any, Ptr{Cvoid}}}()

function plan_for(A, sz::Dims, ::Type{T}) where {T <: Union{Float32, Float64}}
    cache = get!(() -> Dict{Any, Ptr{Cvoid}}(), PLANS, A)
    _cached!(cache, (sz, T), _coeff_key(A), :deo_plan_destroy) do
        gs = _ghosts(A)
        ops = [deo_operator(g.L) for g in gs]
        bcs = [deo_bc(_bc_for(g.Q, _axis(g.L))) for g in gs]
        lines = [_deo_line_bcs(g.Q, _axis(g.L)) for g in gs]
        terms = [DeoTerm(ops[i], _axis(gs[i].L), pointer(bcs, i), C_NULL, 0,
                         lines[i] === nothing ? Ptr{DeoBC}(C_NULL) : pointer(lines[i])) for i in eachindex(gs)]
        sizes = Int64[sz...]
        h = Ref{Ptr{Cvoid}}(C_NULL)
        GC.@preserve bcs lines sizes terms check(ccall((:deo_plan_create, libdeo), Cint,
                                                 (Cint, Ptr{Int64}, Cint, Cint, Ptr{DeoTerm}, Ref{Ptr{Cvoid}}),
                                                 length(sz), sizes, T === Float64 ? 0 : 1, length(terms), terms, h))
        foreach(op -> ccall((:deo_operator_destroy, libdeo), Cvoid, (Ptr{Cvoid},), op), ops)
        h[]
    end
end

_stream() = CUDA.stream().handle

# mul!(du, A*Q, u) and (A*Q)*u on the GPU (ghost_derivative_operator.jl:15-37,
# composite_operators.jl:64-83)
const GhostCombination = DiffEqOperatorCombination{<:Any, <:Tuple{Vararg{GhostDerivativeOperator}}}
const DerivCombination = DiffEqOperatorCombination{<:Any, <:Tuple{Vararg{DerivativeOperator}}}
const DeoOp = Union{GhostDerivativeOperator, GhostCombination}

function _ghost_mul!(du::CuArray{T}, A::DeoOp, u::CuArray{T}, overwrite) where {T <: Union{Float32, Float64}}
    size(du) == size(u) || throw(DimensionMismatch("du and u differ in size"))
    p = plan_for(A, size(u), T)
    check(ccall((:deo_apply, libdeo), Cint, (Ptr{Cvoid}, CuPtr{T}, CuPtr{T}, Cint, Ptr{Cvoid}),
                p, u, du, overwrite, _stream()))
    return du
end

# Every method below is strictly more specific than the reference method it
# shadows (the reference defines each for AbstractVecOrMat and AbstractArray,
# its sums also for 2-D and 3-D arrays), so no call is ambiguous.
const FT = Union{Float32, Float64}
for CA in (:CuVecOrMat, :CuArray)
    @eval begin
        LinearAlgebra.mul!(du::$CA{T}, A::GhostDerivativeOperator, u::$CA{T}; overwrite = true) where {T <: FT} =
            _ghost_mul!(du, A, u, overwrite)
        Base.:*(A::GhostDerivativeOperator, u::$CA{T}) where {T <: FT} = _ghost_mul!(similar(u), A, u, true)
        Base.:*(A::GhostCombination, u::$CA{T}) where {T <: FT} = _ghost_mul!(similar(u), A, u, true)
    end
end
for Nd in 1:3
    @eval LinearAlgebra.mul!(du::CuArray{T, $Nd}, A::GhostCombination, u::CuArray{T, $Nd};
                             overwrite = true) where {T <: FT} = _ghost_mul!(du, A, u, overwrite)
end
LinearAlgebra.mul!(du::CuArray{T}, A::GhostCombination, u::CuArray{T}; overwrite = true) where {T <: FT} =
    _ghost_mul!(du, A, u, overwrite)

# The (L)(du, u, p, t) right-hand-side interface needs no method here: the
# reference's own (DiffEqOperators.jl:67-76) runs update_coefficients! and then
# mul!, which dispatches to the CuArray methods above; the plan caches are keyed
# on the coefficient values, so updated coefficients reach the device.

# ---- L*M and mul!(x_temp, L, M) on an already padded array -------------------
# (derivative_operator_functions.jl:17-69, 150-163; convolutions.jl:17-22), and
# sums of DerivativeOperators on one (composite_operators.jl:64-83 and the
# 2-D / 3-D method of derivative_operator_functions.jl:203-802, whose fallback
# branch -- the one operators with Vector coefficients take -- reads views of
# M that begin at index 1 on the other axes: deo_padded_plan_view)
const PADDED = IdDict{Any, Dict{Any, Ptr{Cvoid}}}()

function padded_plan_for(L::DerivativeOperator, osz::Dims, isz::Dims, ::Type{T},
                         starts) where {T <: Union{Float32, Float64}}
    cache = get!(() -> Dict{Any, Ptr{Cvoid}}(), PADDED, L)
    _cached!(cache, (osz, isz, T, starts), _coeff_key(L), :deo_padded_destroy) do
        op = deo_operator(L)
        o, i = Int64[osz...], Int64[isz...]
        h = Ref{Ptr{Cvoid}}(C_NULL)
        dt = T === Float64 ? 0 : 1
        if starts === nothing
            GC.@preserve o i check(ccall((:deo_padded_plan, libdeo), Cint,
                                         (Ptr{Cvoid}, Cint, Cint, Ptr{Int64}, Ptr{Int64}, Cint, Ref{Ptr{Cvoid}}),
                                         op, _axis(L), length(osz), o, i, dt, h))
        else
            st = Int64[starts...]
            GC.@preserve o i st check(ccall((:deo_padded_plan_view, libdeo), Cint,
                                            (Ptr{Cvoid}, Cint, Cint, Ptr{Int64}, Ptr{Int64}, Ptr{Int64}, Cint,
                                             Ref{Ptr{Cvoid}}), op, _axis(L), length(osz), o, i, st, dt, h))
        end
        ccall((:deo_operator_destroy, libdeo), Cvoid, (Ptr{Cvoid},), op)
        h[]
    end
end

function _padded!(x_temp::CuArray{T}, L::DerivativeOperator, M::CuArray{T}, overwrite::Bool,
                  starts = nothing) where {T <: Union{Float32, Float64}}
    p = padded_plan_for(L, size(x_temp), size(M), T, starts)
    check(ccall((:deo_padded_apply, libdeo), Cint, (Ptr{Cvoid}, CuPtr{T}, CuPtr{T}, Cint, Ptr{Cvoid}),
                p, M, x_temp, overwrite, _stream()))
    return x_temp
end

function _padded_times(L::DerivativeOperator, M::CuArray{T}) where {T <: FT}
    N = _axis(L)
    return _padded!(similar(M, ntuple(b -> b == N ? size(M, b) - 2 : size(M, b), ndims(M))), L, M, true)
end

function _comb_mul!(x_temp::CuArray{T}, A::DerivCombination, M::CuArray{T}) where {T <: FT}
    nd = ndims(M)
    if nd == 1
        for (k, L) in enumerate(A.ops)
            _padded!(x_temp, L, M, k == 1)
        end
        return x_temp
    end
    nd in (2, 3) || throw(MethodError(mul!, (x_temp, A, M)))
    operated = Set(_axis(L) for L in A.ops)
    for (k, L) in enumerate(A.ops)
        others = setdiff(1:nd, (_axis(L),))
        if nd == 2 && isempty(intersect(others, operated))
            _padded!(x_temp, L, M, k == 1)
        else
            _padded!(x_temp, L, M, k == 1, ntuple(_ -> 0, nd))
        end
    end
    return x_temp
end

function _comb_times(A::DerivCombination, M::CuArray{T}) where {T <: FT}
    x = _padded_times(A.ops[1], M)
    for L in A.ops[2:end]
        N = _axis(L)
        sz = ntuple(b -> b == N ? size(M, b) - 2 : size(M, b), ndims(M))
        sz == size(x) || throw(DimensionMismatch("dimensions must match: a has dims $(size(x)), b has dims $sz"))
        _padded!(x, L, M, false)
    end
    return x
end

for CA in (:CuVecOrMat, :CuArray)
    @eval begin
        LinearAlgebra.mul!(x_temp::$CA{T}, L::DerivativeOperator{T, N}, M::$CA{T};
                           overwrite = true) where {T <: FT, N} = _padded!(x_temp, L, M, overwrite)
        Base.:*(L::DerivativeOperator{T, N}, M::$CA{T}) where {T <: FT, N} = _padded_times(L, M)
        Base.:*(A::DerivCombination, M::$CA{T}) where {T <: FT} = _comb_times(A, M)
    end
end
for Nd in 1:3
    @eval LinearAlgebra.mul!(x_temp::CuArray{T, $Nd}, A::DerivCombination, M::CuArray{T, $Nd}) where {T <: FT} =
        _comb_mul!(x_temp, A, M)
end

# ---- ChainRulesCore.rrule: pullback = adjoint kernel ------------------------
using ChainRulesCore
function ChainRulesCore.rrule(::typeof(*), A::DeoOp, u::CuArray{T}) where {T <: Union{Float32, Float64}}
    y = A * u
    p = plan_for(A, size(u), T)
    function pullback(ȳ)
        ū = similar(u)
        ȳc = CuArray{T}(unthunk(ȳ))
        check(ccall((:deo_apply_adjoint, libdeo), Cint, (Ptr{Cvoid}, CuPtr{T}, CuPtr{T}, Cint, Ptr{Cvoid}),
                    p, ȳc, ū, 1, _stream()))
        return NoTangent(), NoTangent(), ū
    end
    return y, pullback
end

# ---- A \ u (ghost_derivative_operator.jl:39-58): banded LU once, every line on the GPU ----
const SOLVES = IdDict{Any, Dict{Any, Ptr{Cvoid}}}()

function solve_plan_for(A::GhostDerivativeOperator, sz::Dims, ::Type{T}) where {T <: Union{Float32, Float64}}
    cache = get!(() -> Dict{Any, Ptr{Cvoid}}(), SOLVES, A)
    _cached!(cache, (sz, T), _coeff_key(A), :deo_solve_destroy) do
        _deo_line_bcs(A.Q, _axis(A.L)) === nothing ||
            throw(ArgumentError("A \\ u is built here for one BC per axis, not an array of per-line BCs"))
        op = deo_operator(A.L)
        bc = Ref(deo_bc(_bc_for(A.Q, _axis(A.L))))
        sizes = Int64[sz...]
        h = Ref{Ptr{Cvoid}}(C_NULL)
        GC.@preserve sizes check(ccall((:deo_solve_plan, libdeo), Cint,
                                       (Ptr{Cvoid}, Ref{DeoBC}, Cint, Ptr{Int64}, Cint, Cint, Ref{Ptr{Cvoid}}),
                                       op, bc, length(sz), sizes, _axis(A.L), T === Float64 ? 0 : 1, h))
        ccall((:deo_operator_destroy, libdeo), Cvoid, (Ptr{Cvoid},), op)
        h[]
    end
end

function _ghost_ldiv(A::GhostDerivativeOperator, u::CuArray{T}) where {T <: FT}
    x = similar(u)
    check(ccall((:deo_solve_apply, libdeo), Cint, (Ptr{Cvoid}, CuPtr{T}, CuPtr{T}, Ptr{Cvoid}),
                solve_plan_for(A, size(u), T), u, x, _stream()))
    return x
end
# the reference defines \ for AbstractVector, AbstractMatrix and AbstractArray
Base.:\(A::GhostDerivativeOperator, u::CuVector{T}) where {T <: FT} = _ghost_ldiv(A, u)
Base.:\(A::GhostDerivativeOperator, u::CuMatrix{T}) where {T <: FT} = _ghost_ldiv(A, u)
Base.:\(A::GhostDerivativeOperator, u::CuArray{T}) where {T <: FT} = _ghost_ldiv(A, u)

# ---- vector calculus (vector_calculus_operators.jl, vector_calculus_convolutions.jl) ----
const VC_PLANS = IdDict{Any, Dict{Any, Ptr{Cvoid}}}()
_vc_kind(::GradientOperator) = 0
_vc_kind(::DivergenceOperator) = 1
_vc_kind(::CurlOperator) = 2
const DeoVC = Union{GradientOperator, DivergenceOperator, CurlOperator}

function vc_plan_for(A::DeoVC, ::Type{T}) where {T <: Union{Float32, Float64}}
    cache = get!(() -> Dict{Any, Ptr{Cvoid}}(), VC_PLANS, A)
    _cached!(cache, T, hash(map(_coeff_key, vec(A.ops))), :deo_vector_calculus_destroy) do
        ops = [deo_operator(L) for L in vec(A.ops)]
        h = Ref{Ptr{Cvoid}}(C_NULL)
        GC.@preserve ops check(ccall((:deo_vector_calculus_plan, libdeo), Cint,
                                     (Cint, Cint, Ptr{Ptr{Cvoid}}, Cint, Ref{Ptr{Cvoid}}),
                                     _vc_kind(A), length(ops), ops, T === Float64 ? 0 : 1, h))
        foreach(op -> ccall((:deo_operator_destroy, libdeo), Cvoid, (Ptr{Cvoid},), op), ops)
        h[]
    end
end

function _vc_apply!(x_temp::CuArray{T}, A::DeoVC, M::CuArray{T}, overwrite) where {T <: Union{Float32, Float64}}
    check(ccall((:deo_vector_calculus_apply, libdeo), Cint, (Ptr{Cvoid}, CuPtr{T}, CuPtr{T}, Cint, Ptr{Cvoid}),
                vc_plan_for(A, T), M, x_temp, overwrite, _stream()))
    return x_temp
end

# mul! accumulates, as the reference's methods do; the 2-D and 3-D methods
# shadow the reference's own dimension-specific ones
LinearAlgebra.mul!(x_temp::CuArray{T}, has_vector::Bool, A::Union{GradientOperator, DivergenceOperator},
                   M::CuArray{T}; overwrite = false) where {T <: FT} = _vc_apply!(x_temp, A, M, 0)
for MT in (2, 3)
    @eval LinearAlgebra.mul!(x_temp::CuArray{T}, has_vector::Bool,
                             A::Union{GradientOperator{T, $MT}, DivergenceOperator{T, $MT}},
                             M::CuArray{T}; overwrite = false) where {T <: FT} = _vc_apply!(x_temp, A, M, 0)
end
LinearAlgebra.mul!(x_temp::CuArray{T, 4}, A::CurlOperator, M::CuArray{T, 4};
                   overwrite = false) where {T <: FT} = _vc_apply!(x_temp, A, M, 0)

function Base.:*(A::GradientOperator{T}, M::CuArray{T, N}) where {T <: FT, N}
    _vc_apply!(CuArray{T}(undef, (size(M) .- 2)..., N), A, M, 1)
end
function Base.:*(A::DivergenceOperator{T}, M::CuArray{T, N}) where {T <: FT, N}
    _vc_apply!(CuArray{T}(undef, (size(M)[1:(end - 1)] .- 2)...), A, M, 1)
end
function Base.:*(A::CurlOperator{T}, M::CuArray{T, 4}) where {T <: FT}
    _vc_apply!(CuArray{T}(undef, (size(M)[1:3] .- 2)..., 3), A, M, 1)
end

# ---- BandedMatrix(A*Q) from the device (concretization.jl:926-936) ----------
using BandedMatrices: _BandedMatrix

"""device_banded(A, sz, T) -> (BandedMatrix A_l, A_b): the affine map of the
GhostDerivativeOperator (or combination) A on arrays of size sz, built on the
device from the plan's row tables (deo_plan_concretize_banded)."""
function device_banded(A::DeoOp, sz::Dims, ::Type{T} = Float64) where {T <: FT}
    p = plan_for(A, sz, T)
    l, u = Ref{Int64}(0), Ref{Int64}(0)
    check(ccall((:deo_plan_bandwidths, libdeo), Cint, (Ptr{Cvoid}, Ref{Int64}, Ref{Int64}, Ptr{Cvoid}),
                p, l, u, _stream()))
    n = prod(sz)
    data = CuArray{Float64}(undef, l[] + u[] + 1, n)
    Ab = CuArray{Float64}(undef, n)
    check(ccall((:deo_plan_concretize_banded, libdeo), Cint,
                (Ptr{Cvoid}, Int64, Int64, CuPtr{Float64}, CuPtr{Float64}, Ptr{Cvoid}), p, l[], u[], data, Ab, _stream()))
    return _BandedMatrix(Array(data), n, l[], u[]), Array(Ab)
end

# ---- serving (deo_serve_*): MOL solves of (L)(du,u,p,t) = mul!(du, L, u) ----
# Each request: K SSP-RK3 steps of du/dt = A*Q*u from a host array u0 (and,
# with want_grad, the gradient of ||u(T)||^2 with respect to u0).  The server
# keeps admitted states on the device under its byte budget; `pump!` never
# waits for the device.
struct DeoRequest
    plan::Ptr{Cvoid}
    u0::Ptr{Cvoid}
    nsteps::Cint
    dt::Cdouble
    want_grad::Cint
end

mutable struct DeoServer
    h::Ptr{Cvoid}
    T::DataType
    inputs::Dict{Int64, Any}   # u0 kept alive until the submission has copied it
end

function DeoServer(budget_bytes::Integer, ::Type{T} = Float64; max_steps_per_round::Integer = 64) where {T <: FT}
    h = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:deo_serve_create, libdeo), Cint, (Csize_t, Cint, Cint, Ref{Ptr{Cvoid}}),
                budget_bytes, T === Float64 ? 0 : 1, max_steps_per_round, h))
    s = DeoServer(h[], T, Dict{Int64, Any}())
    finalizer(x -> ccall((:deo_serve_destroy, libdeo), Cvoid, (Ptr{Cvoid},), x.h), s)
    return s
end

"""submit!(s, A, u0, K, dt; want_grad=false) -> request id (an `ErrorException`
carries DEO_ERR_REJECTED when the state is larger than the budget)."""
function submit!(s::DeoServer, A::DeoOp, u0::Array{T}, K::Integer, dt::Real; want_grad::Bool = false) where {T <: FT}
    T === s.T || throw(ArgumentError("the server serves $(s.T)"))
    p = plan_for(A, size(u0), T)
    rid = Ref{Int64}(0)
    q = Ref(DeoRequest(p, pointer(u0), K, dt, want_grad))
    GC.@preserve u0 check(ccall((:deo_serve_submit, libdeo), Cint, (Ptr{Cvoid}, Ref{DeoRequest}, Ref{Int64}),
                                s.h, q, rid))
    return rid[]
end

pump!(s::DeoServer) = check(ccall((:deo_serve_pump, libdeo), Cint, (Ptr{Cvoid},), s.h))

"""poll!(s, rid, uT[, grad]) -> true once the result is in uT (and grad), false while it runs."""
function poll!(s::DeoServer, rid::Integer, uT::Array{T}, grad::Union{Nothing, Array{T}} = nothing) where {T <: FT}
    st = GC.@preserve uT grad ccall((:deo_serve_poll, libdeo), Cint,
                                     (Ptr{Cvoid}, Int64, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cdouble}),
                                     s.h, rid, pointer(uT), grad === nothing ? C_NULL : pointer(grad), C_NULL)
    st == 7 && return false   # DEO_ERR_NOT_READY
    check(st)
    return true
end

cancel!(s::DeoServer, rid::Integer) = check(ccall((:deo_serve_cancel, libdeo), Cint, (Ptr{Cvoid}, Int64), s.h, rid))

end # module
