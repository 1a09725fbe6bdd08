# KronFreeGB300: the reference-side binding of libkfgpu.so for KronFreeCircuits.jl.
#
# A custom solver in the reference's documented contract (src/solvers.jl:6-31): `solve(s, H, m; X0)`
# returns host (E, V) and every residual is checked against the operator.  The operator's data is
# handed to the library through the C ABI of include/kfgpu.h; the tree, materialize and ports stay
# unchanged, and a node opts in with `Node(...; solver=GB300(LOBPCG(...)))`.
#
# Usage:
#     using KronFreeCircuits, KronFreeGB300
#     KronFreeGB300.load("/path/to/libkfgpu.so")
#     leaf = Node([...]; solver=GB300Solver(kind=:lobpcg, precision=:mixed, preconditioner=:separable))
module KronFreeGB300

using KronFreeCircuits
using KronFreeCircuits: KronFreeOperator, DenseOp, DiagonalOp, BandedOp, ShiftOp
import KronFreeCircuits: solve, storage

const LIB = Ref{String}("libkfgpu.so")
load(path::AbstractString) = (LIB[] = path; nothing)

# ---- C structs (include/kfgpu.h) ------------------------------------------------------------
struct KfFactor
    axis::Int32; kind::Int32; n::Int64
    data::Ptr{Float64}; offsets::Ptr{Int64}; nbands::Int32
    shift::Int64; factor::Float64
end
struct KfTerm
    coeff::Float64; nfactors::Int32; factors::Ptr{KfFactor}
end
struct KfOpDesc
    ndims::Int32; dims::Ptr{Int64}; constant::Float64
    nterms::Int32; terms::Ptr{KfTerm}; diag::Ptr{Float64}; block_capacity::Int64
end
mutable struct KfSolverOpts
    kind::Int32; precision::Int32; tol::Float64; maxiter::Int32; preconditioner::Int32; eta::Float64
    guard::Int32; degree::Int32; extra::Int32; rescale_every::Int32; ortho::Int32; bound::Float64
    krylovdim::Int32; rng_seed::UInt64; mixed_switch::Float64; fallback_iters::Int32; fallback_resid::Float64
    seed_kind::Int32; buffer::Int32
    KfSolverOpts() = new()
end
mutable struct KfSolveStats
    iterations::Int32; iterations_f64::Int32; n_matvec::Int64; warm::Int32; fell_back::Int32; converged::Int32
    max_residual::Float64; hnorm::Float64; seconds::Float64; seconds_f64::Float64
    KfSolveStats() = new()
end

const KF_OK, KF_EINVAL, KF_EDIM, KF_EALIAS = 0, 1, 2, 3
const KF_ENOCONV, KF_EBREAKDOWN, KF_ENOTFINITE = 5, 6, 9

function _check(status)
    status == KF_OK && return nothing
    buf = Vector{UInt8}(undef, 4096)
    ccall((:kf_last_error, LIB[]), Cint, (Ptr{UInt8}, Csize_t), buf, length(buf))
    msg = unsafe_string(pointer(buf))
    status in (KF_EINVAL, KF_EALIAS) && throw(ArgumentError(msg))
    status == KF_EDIM && throw(DimensionMismatch(msg))
    error(msg)
end

# The descriptor of a real KronFreeOperator: every fused term (H.diagterms, the constant as a
# zero-factor term) and every kept term (H.terms), 0-based axes; `keep` holds what the pointers
# point into until the call returns.
function _descriptor(H::KronFreeOperator, keep::Vector{Any})
    eltype(H) <: Real || throw(ArgumentError("KronFreeGB300: real operators only (eltype $(eltype(H)))"))
    function cfactor(a, op)
        if op isa DiagonalOp
            d = Vector{Float64}(op.d); push!(keep, d)
            return KfFactor(a - 1, 0, length(d), pointer(d), C_NULL, 0, 0, 0.0)
        elseif op isa BandedOp
            w = reduce(vcat, Vector{Float64}.(op.weights); init=Float64[]); o = Vector{Int64}(op.offsets)
            push!(keep, w); push!(keep, o)
            return KfFactor(a - 1, 1, op.n, pointer(w), pointer(o), length(o), 0, 0.0)
        elseif op isa ShiftOp
            return KfFactor(a - 1, 2, op.n, C_NULL, C_NULL, 0, op.s, Float64(op.factor))
        else
            M = Matrix{Float64}(op.M); push!(keep, M)
            return KfFactor(a - 1, 3, size(M, 1), pointer(M), C_NULL, 0, 0, 0.0)
        end
    end
    terms = KfTerm[]
    for t in H.diagterms
        fs = KfFactor[cfactor(a, op) for (a, op) in t.factors]; push!(keep, fs)
        push!(terms, KfTerm(Float64(t.coeff), length(fs), pointer(fs)))
    end
    for t in H.terms
        fs = KfFactor[cfactor(a, op) for (a, op, _) in t.factors]; push!(keep, fs)
        push!(terms, KfTerm(Float64(t.coeff), length(fs), pointer(fs)))
    end
    dims = Vector{Int64}(H.dims); push!(keep, dims); push!(keep, terms)
    return Ref(KfOpDesc(length(dims), pointer(dims), 0.0, length(terms), pointer(terms), C_NULL,
                        max(1, KronFreeCircuits._block_capacity(H))))
end

"""
    GB300Solver(; kind=:lobpcg, precision=:mixed, preconditioner=:separable, tol=1e-8, maxiter=1000,
                eta=0.01, guard=4, seed=:product, degree=100, extra=40, krylovdim=0)

A solver for `Node(...; solver=...)` that runs on one GB300 through libkfgpu.so: LOBPCG
(src/lobpcg.jl), ChebyshevFilter (src/chebyshev.jl) or Lanczos (src/solvers.jl:85-106), with the
reference's options plus `precision` (`:f64` or `:mixed`) and the `:separable` preconditioner.
Results are host arrays; `storage(s)` is `Array` because the operator is copied by the library.
"""
Base.@kwdef struct GB300Solver <: KronFreeCircuits.Solver
    kind::Symbol = :lobpcg
    precision::Symbol = :mixed
    preconditioner::Symbol = :separable
    tol::Float64 = 1e-8
    maxiter::Int = 1000
    eta::Float64 = 0.01
    guard::Int = 4
    seed::Symbol = :product
    degree::Int = 100
    extra::Int = 40
    krylovdim::Int = 0
end

storage(::GB300Solver) = Array

function solve(s::GB300Solver, H::KronFreeOperator, m::Int; X0=nothing)
    keep = Any[]
    desc = _descriptor(H, keep)
    op = Ref{Ptr{Cvoid}}(C_NULL)
    GC.@preserve keep begin
        _check(ccall((:kf_op_create, LIB[]), Cint, (Ref{KfOpDesc}, Ref{Ptr{Cvoid}}), desc, op))
    end
    try
        kind = Int32(s.kind === :lobpcg ? 0 : s.kind === :chebyshev ? 1 : 2)
        o = KfSolverOpts()
        ccall((:kf_solver_opts_default, LIB[]), Cvoid, (Ref{KfSolverOpts}, Int32), o, kind)
        o.precision = s.precision === :mixed ? 1 : 0
        o.tol, o.maxiter, o.eta, o.guard = s.tol, s.maxiter, s.eta, s.guard
        o.preconditioner = Dict(:ritz => 0, :jacobi => 1, :none => 2, :separable => 3)[s.preconditioner]
        o.degree, o.extra, o.krylovdim = s.degree, s.extra, s.krylovdim
        N = size(H, 1)
        # seed=:product: the library builds product_seed(H, w) on the device (kf_op_product_seed)
        o.seed_kind = s.seed === :product ? 0 : 1
        seed = nothing
        x0 = X0 === nothing ? nothing : Matrix{Float64}(X0)
        E = Vector{Float64}(undef, m); V = Matrix{Float64}(undef, N, m); st = KfSolveStats()
        _check(ccall((:kf_solve, LIB[]), Cint,
                     (Ptr{Cvoid}, Ref{KfSolverOpts}, Int32, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64},
                      Ref{KfSolveStats}),
                     op[], o, m, x0 === nothing ? C_NULL : x0, seed === nothing ? C_NULL : seed, E, V, st))
        return E, V
    finally
        ccall((:kf_op_destroy, LIB[]), Cint, (Ptr{Cvoid},), op[])
    end
end

end # module
