"""
    SymmetricEigenProblemGB300

Julia binding of libsymeig.so: the GB300 implementation of SymmetricEigenProblem.jl's
eigensolver hot path.  The functions keep the reference's names and signatures:

    qr_algorithm!(H::SymTridiagonal{Float64}, Q, max_layers=128, tol=eps(Float64), maxiter=100n)
        -> (H, converged::Bool, iter::Int)                      # src/bulge_chasing.jl:146
    bulk_wave_order_2x2_rmul!(A, givens::Matrix{Tuple{T,T}})   # src/wave.jl:62
    bulk_wave_order_2x2_rmul_parallel!(A, givens)              # src/wave.jl:36
    eigen_decomp!(H) -> (Diagonal(H.dv), Q)                    # src/bulge_chasing.jl:290

Q may be Matrix{Float64} or Matrix{Float32} (the FP32-Q variant: FP64 chase, (c,s) rounded to
Float32).  Host arrays are copied to the GPU and back by the library.  Nothing is exported,
as in the reference.  Unlike the reference, odd n is accepted.
"""
module SymmetricEigenProblemGB300

using LinearAlgebra: SymTridiagonal, Diagonal, I

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

function eigen_decomp!(H::SymTridiagonal{Float64})
    n = size(H, 1)
    Q = Matrix{Float64}(I, n, n)
    _, converged, iter = qr_algorithm!(H, Q)
    @info "done" converged iter
    return Diagonal(H.dv), Q
end

end # module
