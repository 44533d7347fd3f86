"""
    SymmetricEigenProblemGB300

Julia binding of libsymeig.so: the GB300 implementation of SymmetricEigenProblem.jl's
eigensolver hot path.  The functions keep the reference's names and signatures:

    qr_algorithm!(H::SymTridiagonal{Float64}, Q, max_layers=128, tol=eps(Float64), maxiter=100n)
        -> (H, converged::Bool, iter::Int)                      # src/bulge_chasing.jl:146
    bulk_wave_order_2x2_rmul!(A, givens::Matrix{Tuple{T,T}})   # src/wave.jl:62
    bulk_wave_order_2x2_rmul_parallel!(A, givens)              # src/wave.jl:36
    eigen_decomp!(H) -> (Diagonal(H.dv), Q)                    # src/bulge_chasing.jl:290

and three additions without a reference counterpart:

    qr_algorithm_batched!(Hs::Vector{SymTridiagonal{Float64}}, Qs; max_layers, tol, maxiter_factor)
    tridiag_eigen(d, e) -> (lam, Q), differentiable through a ChainRulesCore rrule whose
        pullback is the library's adjoint (FP64 tensor-core GEMMs with fused epilogues)
    bulk_wave_order_2x2_lmul!(A, givens)                      # bulk form of lmul!, src/simple_givens.jl:38
    get_rotation(f, g) -> (c, s, r), elementwise               # src/simple_givens.jl:20
    syev!(A) -> (lam, V): dense symmetric eigensolve (sytrd, orgtr, qr_algorithm!)
    set_apply_form!(form), set_chase_mode!(mode), set_multishift!(bulges, rows, release),
    set_multishift_min!(bulges):
        the library's arithmetic options (chase mode 3 is the multishift chase)

Q may be Matrix{Float64} or Matrix{Float32} (the FP32-Q variant: FP64 chase, (c,s) rounded to
Float32).  Host arrays are copied to the GPU and back by the library.  Nothing is exported,
as in the reference.  Unlike the reference, odd n is accepted.
"""
module SymmetricEigenProblemGB300

import LinearAlgebra
using LinearAlgebra: SymTridiagonal, Diagonal, I
using ChainRulesCore: ChainRulesCore, NoTangent, AbstractZero, unthunk

const libsymeig = get(ENV, "SYMEIG_LIB",
                      joinpath(@__DIR__, "..", "_build", "libsymeig.so"))

struct SymeigError <: Exception
    fn::Symbol
    status::Cint
end
Base.showerror(io::IO, e::SymeigError) =
    print(io, e.fn, " failed: ", unsafe_string(ccall((:symeig_status_string, libsymeig), Cstring, (Cint,), e.status)))

check(fn::Symbol, st::Cint) = st == 0 ? nothing : throw(SymeigError(fn, st))

# One handle per Julia thread (handles are not shared across threads).
const HANDLES = Dict{Int,Ptr{Cvoid}}()
const HANDLE_LOCK = ReentrantLock()
function handle()
    tid = Threads.threadid()
    lock(HANDLE_LOCK) do
        get!(HANDLES, tid) do
            h = Ref{Ptr{Cvoid}}(C_NULL)
            check(:symeig_create, ccall((:symeig_create, libsymeig), Cint, (Ref{Ptr{Cvoid}}, Cint), h, 0))
            h[]
        end
    end
end

function qr_algorithm!(H::SymTridiagonal{Float64}, Q::StridedMatrix{T}, max_layers::Int = 128,
                       tol = eps(Float64), maxiter::Int = 100 * size(H, 1)) where {T<:Union{Float64,Float32}}
    n = size(H, 1)
    size(Q, 2) == n || throw(DimensionMismatch("Q must have n columns"))
    stride(Q, 1) == 1 || throw(ArgumentError("Q must have unit row stride"))
    conv = Ref{Int32}(0)
    iter = Ref{Int64}(0)
    fn = T === Float64 ? :symeig_qr_f64 : :symeig_qr_f64_q32
    st = GC.@preserve H Q ccall((fn, libsymeig), Cint,
        (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Int64, Ptr{T}, Int64, Int64, Int32, Float64, Int64,
         Ref{Int32}, Ref{Int64}),
        handle(), H.dv, H.ev, n, Q, stride(Q, 2), size(Q, 1), max_layers, Float64(tol), maxiter,
        conv, iter)
    check(fn, st)
    return H, conv[] != 0, Int(iter[])
end

function bulk_wave_order_2x2_rmul!(A::StridedMatrix{T}, givens::Matrix{Tuple{T,T}}) where {T<:Union{Float64,Float32}}
    m, n = size(A)
    size(givens, 1) == n - 1 || throw(DimensionMismatch("givens must have n-1 rows"))
    stride(A, 1) == 1 || throw(ArgumentError("A must have unit row stride"))
    fn = T === Float64 ? :symeig_apply_givens_f64 : :symeig_apply_givens_f32
    # Matrix{Tuple{T,T}} is stored as interleaved (c, s) pairs, column-major: the C layout
    st = GC.@preserve A givens ccall((fn, libsymeig), Cint,
        (Ptr{Cvoid}, Ptr{T}, Int64, Int64, Int64, Ptr{Tuple{T,T}}, Int64),
        handle(), A, stride(A, 2), m, n, givens, size(givens, 2))
    check(fn, st)
    return nothing
end

# Every row of A has its own GPU thread: the threaded variant is the same call.
bulk_wave_order_2x2_rmul_parallel!(A, givens) = bulk_wave_order_2x2_rmul!(A, givens)

function bulk_wave_order_2x2_lmul!(A::StridedMatrix{T}, givens::Matrix{Tuple{T,T}}) where {T<:Union{Float64,Float32}}
    m, n = size(A)
    size(givens, 1) == m - 1 || throw(DimensionMismatch("givens must have m-1 rows"))
    stride(A, 1) == 1 || throw(ArgumentError("A must have unit row stride"))
    fn = T === Float64 ? :symeig_apply_givens_left_f64 : :symeig_apply_givens_left_f32
    st = GC.@preserve A givens ccall((fn, libsymeig), Cint,
        (Ptr{Cvoid}, Ptr{T}, Int64, Int64, Int64, Ptr{Tuple{T,T}}, Int64),
        handle(), A, stride(A, 2), m, n, givens, size(givens, 2))
    check(fn, st)
    return nothing
end

"""Many qr_algorithm! calls in one: H_i and Q_i (n_i x n_i) updated in place.  Q_i are all
Float64, or all Float32 (the FP32-Q variant: the chase stays Float64)."""
function qr_algorithm_batched!(Hs::Vector{SymTridiagonal{Float64,Vector{Float64}}}, Qs::Vector{Matrix{T}};
                               max_layers::Int = 128, tol = eps(Float64),
                               maxiter_factor::Int = 100) where {T<:Union{Float32,Float64}}
    ns = Int64[size(H, 1) for H in Hs]
    d = reduce(vcat, [H.dv for H in Hs])
    e = reduce(vcat, [H.ev for H in Hs])
    Q = reduce(vcat, [vec(Q) for Q in Qs])
    conv = zeros(Int32, length(Hs))
    iters = zeros(Int64, length(Hs))
    if T === Float64
        st = ccall((:symeig_qr_batched_f64, libsymeig), Cint,
            (Ptr{Cvoid}, Int64, Ptr{Int64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Int32, Float64, Int64,
             Ptr{Int32}, Ptr{Int64}),
            handle(), length(Hs), ns, d, e, Q, max_layers, Float64(tol), maxiter_factor, conv, iters)
        check(:symeig_qr_batched_f64, st)
    else
        st = ccall((:symeig_qr_batched_f64_q32, libsymeig), Cint,
            (Ptr{Cvoid}, Int64, Ptr{Int64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float32}, Int32, Float64, Int64,
             Ptr{Int32}, Ptr{Int64}),
            handle(), length(Hs), ns, d, e, Q, max_layers, Float64(tol), maxiter_factor, conv, iters)
        check(:symeig_qr_batched_f64_q32, st)
    end
    od = oe = oq = 0
    for (k, n) in enumerate(ns)
        Hs[k].dv .= view(d, od+1:od+n); od += n
        Hs[k].ev .= view(e, oe+1:oe+n-1); oe += n - 1
        vec(Qs[k]) .= view(Q, oq+1:oq+n*n); oq += n * n
    end
    return Hs, conv .!= 0, iters
end

"""(lam, Q) of SymTridiagonal(d, e): lam unsorted (as H.dv), Q the eigenvectors."""
function tridiag_eigen(d::AbstractVector{Float64}, e::AbstractVector{Float64})
    n = length(d)
    H = SymTridiagonal(collect(d), collect(e))
    Q = Matrix{Float64}(I, n, n)
    _, converged, _ = qr_algorithm!(H, Q)
    converged || error("qr_algorithm! did not converge")
    return H.dv, Q
end

function ChainRulesCore.rrule(::typeof(tridiag_eigen), d::AbstractVector{Float64}, e::AbstractVector{Float64})
    lam, Q = tridiag_eigen(d, e)
    n = length(d)
    function tridiag_eigen_pullback(ybar)
        glam_t, gQ_t = unthunk(ybar)
        glam = glam_t isa AbstractZero ? zeros(n) : collect(Float64, unthunk(glam_t))
        gQ = gQ_t isa AbstractZero ? nothing : Matrix{Float64}(unthunk(gQ_t))
        gd = zeros(n)
        ge = zeros(max(n - 1, 0))
        st = GC.@preserve lam Q glam gQ ccall((:symeig_eig_adjoint_f64, libsymeig), Cint,
            (Ptr{Cvoid}, Int64, Int64, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64},
             Ptr{Float64}, Ptr{Float64}),
            handle(), 1, n, lam, Q, glam, gQ === nothing ? C_NULL : gQ, gd, ge)
        check(:symeig_eig_adjoint_f64, st)
        return NoTangent(), gd, ge
    end
    return (lam, Q), tridiag_eigen_pullback
end

"""Elementwise get_rotation (LinearAlgebra.givensAlgorithm) computed on the device."""
function get_rotation(f::Vector{Float64}, g::Vector{Float64})
    length(f) == length(g) || throw(DimensionMismatch("f and g must have one length"))
    c, s, r = similar(f), similar(f), similar(f)
    st = ccall((:symeig_get_rotation_f64, libsymeig), Cint,
        (Ptr{Cvoid}, Int64, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}),
        handle(), length(f), f, g, c, s, r)
    check(:symeig_get_rotation_f64, st)
    return c, s, r
end

"""Dense symmetric eigensolve: (lam, V) with lam unsorted (as H.dv) and V the eigenvectors.
A is left unchanged (the library copies it to the device)."""
function syev!(A::StridedMatrix{Float64})
    n = LinearAlgebra.checksquare(A)
    stride(A, 1) == 1 || throw(ArgumentError("A must have unit row stride"))
    lam = Vector{Float64}(undef, n)
    V = Matrix{Float64}(undef, n, n)
    conv = Ref{Int32}(0)
    iter = Ref{Int64}(0)
    st = GC.@preserve A ccall((:symeig_syev_f64, libsymeig), Cint,
        (Ptr{Cvoid}, Int64, Ptr{Float64}, Int64, Ptr{Float64}, Ptr{Float64}, Int64, Ref{Int32}, Ref{Int64}),
        handle(), n, A, stride(A, 2), lam, V, n, conv, iter)
    check(:symeig_syev_f64, st)
    conv[] != 0 || @warn "qr_algorithm! did not converge" iter[]
    return lam, V
end

"""0: canonical rotations (default); 1: the scaled form of the FP64 bulk apply."""
set_apply_form!(form::Integer) =
    check(:symeig_set_apply_form, ccall((:symeig_set_apply_form, libsymeig), Cint, (Ptr{Cvoid}, Int32), handle(), form))

"""0: Newton-form two-warp chase (default); 1: reference form; 2: Newton form with every
sweep redone in the reference form -- these three give the reference's bits.  3: multishift
batches of concurrent bulges (within the reference's error bounds, not its bits; about 8x
faster at n = 16384)."""
set_chase_mode!(mode::Integer) =
    check(:symeig_set_chase_mode, ccall((:symeig_set_chase_mode, libsymeig), Cint, (Ptr{Cvoid}, Int32), handle(), mode))

"""Batch shape of chase mode 3: at most `bulges` (2..128, default 64) bulges per batch, one per
`rows` (default 16) rows of the block, each releasing its progress every `release` steps
(a power of two, default 4)."""
set_multishift!(bulges::Integer = 64, rows::Integer = 16, release::Integer = 4) =
    check(:symeig_set_multishift, ccall((:symeig_set_multishift, libsymeig), Cint,
          (Ptr{Cvoid}, Int32, Int32, Int32), handle(), bulges, rows, release))

"""Fewest bulges of a chase-mode-3 batch (2..128, default 2): a block with room for fewer takes
single sweeps with the reference's shift."""
set_multishift_min!(bulges::Integer = 2) =
    check(:symeig_set_multishift_min, ccall((:symeig_set_multishift_min, libsymeig), Cint,
          (Ptr{Cvoid}, Int32), handle(), bulges))

function eigen_decomp!(H::SymTridiagonal{Float64})
    n = size(H, 1)
    Q = Matrix{Float64}(I, n, n)
    _, converged, iter = qr_algorithm!(H, Q)
    @info "done" converged iter
    return Diagonal(H.dv), Q
end

end # module
