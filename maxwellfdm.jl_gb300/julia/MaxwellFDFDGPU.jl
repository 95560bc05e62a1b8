# MaxwellFDFDGPU — ccall binding of libfdfd_gb300 for MaxwellFDFD.jl.
#
# A GPU operator type that is a drop-in for the SparseMatrixCSC that
# MaxwellFDFD.create_A returns (src/model/model.jl:225-246): it implements
# size, eltype, mul!, *, transpose-mul, ldiv!/\ (GPU Krylov solve) and a
# ChainRulesCore.rrule for the solve with respect to ε and b.  Signatures
# mirror include/fdfd_gb300.h one for one.
module MaxwellFDFDGPU

using LinearAlgebra
using MaxwellFDFD
import ChainRulesCore
using ChainRulesCore: NoTangent, unthunk

export FDFDOperator, create_A_gpu, SolveOpts, eps_grad, h_from_e, e_from_h, corner_mean, solve_with_eps,
       residual_dev!, residual_dev_noalloc!

const libfdfd = joinpath(@__DIR__, "..", "libfdfd_gb300.so")

struct FDFDDesc
    N::NTuple{3,Int32}
    isbloch::NTuple{3,Int32}
    boundft::NTuple{3,Int32}
    order_cmpfirst::Int32
    device::Int32
    slice2d::Int32
    omega::NTuple{2,Float64}
    e_ikl::NTuple{6,Float64}
    sdl_e::NTuple{3,Ptr{Float64}}
    sdl_m::NTuple{3,Ptr{Float64}}
end

Base.@kwdef struct SolveOpts
    method::Int32 = 2          # 0 BiCGSTAB, 1 COCG (FP64 only), 2 BiCGStab(ℓ) (default)
    precision::Int32 = 1       # 0 FP64, 1 mixed (complex64 + FP64 reliable updates)
    tol::Float64 = 1e-6
    maxit::Int64 = 200000
    delta::Float64 = 0.1
    x0_given::Int32 = 0
    check_every::Int32 = 50
    transpose::Int32 = 0
    use_graph::Int32 = 1
    ell::Int32 = 4             # ℓ of BiCGStab(ℓ)
end

struct SolveStats
    iterations::Int64
    matvecs::Int64
    refinements::Int32
    status::Int32
    relres::Float64
    time_ms::Float64
    launches::Int64
end

struct FDFDError <: Exception
    code::Int32
    msg::String
end

function check(rc::Integer, h::Ptr{Cvoid})
    rc == 0 && return nothing
    msg = unsafe_string(ccall((:fdfd_last_error, libfdfd), Cstring, (Ptr{Cvoid},), h))
    throw(FDFDError(rc, msg))
end

mutable struct FDFDOperator <: AbstractMatrix{ComplexF64}
    h::Ptr{Cvoid}
    n::Int
    N::NTuple{3,Int}
    ω::ComplexF64
end

Base.size(A::FDFDOperator) = (A.n, A.n)
Base.eltype(::FDFDOperator) = ComplexF64
Base.getindex(::FDFDOperator, ::Int, ::Int) = error("FDFDOperator is matrix-free")

function create_A_gpu(mdl::MaxwellFDFD.ModelFull, ω::Number; device::Integer=0)
    s∆lₑ, s∆lₘ, _, _ = MaxwellFDFD.create_stretched_∆ls(mdl)
    se = [ComplexF64.(s∆lₑ[w]) for w = 1:3]
    sm = [ComplexF64.(s∆lₘ[w]) for w = 1:3]
    eikl = MaxwellFDFD.create_e⁻ⁱᵏᴸ(mdl)
    N = Tuple(mdl.grid.N)
    d = FDFDDesc(Int32.(N), Int32.(Tuple(mdl.grid.isbloch)), (0, 0, 0), 1, Int32(device), 0,
                 (Float64(real(ω)), Float64(imag(ω))),
                 Tuple(Float64[x for p in eikl for x in (real(p), imag(p))]),
                 Tuple(Ptr{Float64}.(pointer.(se))), Tuple(Ptr{Float64}.(pointer.(sm))))
    h = Ref{Ptr{Cvoid}}(C_NULL)
    GC.@preserve se sm begin
        check(ccall((:fdfd_create, libfdfd), Cint, (Ref{FDFDDesc}, Ref{Ptr{Cvoid}}), d, h), C_NULL)
    end
    A = FDFDOperator(h[], 3prod(N), N, ComplexF64(ω))
    finalizer(A -> ccall((:fdfd_destroy, libfdfd), Cvoid, (Ptr{Cvoid},), A.h), A)
    MaxwellFDFD.calc_matparams!(mdl)
    check(ccall((:fdfd_set_eps_tensor, libfdfd), Cint, (Ptr{Cvoid}, Ptr{ComplexF64}), A.h, mdl.εarr), A.h)
    return A
end

function LinearAlgebra.mul!(y::Vector{ComplexF64}, A::FDFDOperator, x::Vector{ComplexF64})
    check(ccall((:fdfd_matvec, libfdfd), Cint, (Ptr{Cvoid}, Ptr{ComplexF64}, Ptr{ComplexF64}, Int32),
                A.h, x, y, 0), A.h)
    return y
end
Base.:*(A::FDFDOperator, x::Vector{ComplexF64}) = mul!(similar(x), A, x)

function LinearAlgebra.mul!(y::Vector{ComplexF64}, At::Transpose{ComplexF64,FDFDOperator}, x::Vector{ComplexF64})
    check(ccall((:fdfd_matvec_transpose, libfdfd), Cint, (Ptr{Cvoid}, Ptr{ComplexF64}, Ptr{ComplexF64}, Int32),
                parent(At).h, x, y, 0), parent(At).h)
    return y
end

function solve!(x::Vector{ComplexF64}, A::FDFDOperator, b::Vector{ComplexF64}; opts::SolveOpts=SolveOpts())
    st = Ref{SolveStats}()
    check(ccall((:fdfd_solve, libfdfd), Cint,
                (Ptr{Cvoid}, Ptr{ComplexF64}, Ptr{ComplexF64}, Int32, Ref{SolveOpts}, Ref{SolveStats}),
                A.h, b, x, 1, opts, st), A.h)
    return x, st[]
end

LinearAlgebra.ldiv!(x::Vector{ComplexF64}, A::FDFDOperator, b::Vector{ComplexF64}) = first(solve!(x, A, b))
Base.:\(A::FDFDOperator, b::Vector{ComplexF64}) = ldiv!(zeros(ComplexF64, length(b)), A, b)

# Adjoint of e = A \ b for a real objective L(e): with g = ∂L/∂e (Wirtinger
# derivative, dL = 2Re(gᵀde)), λ solves transpose(A) λ = g on the GPU.
function solve_pullback(A::FDFDOperator, e::Vector{ComplexF64}, g::Vector{ComplexF64}; opts::SolveOpts=SolveOpts())
    λ = zeros(ComplexF64, length(g))
    o = SolveOpts(opts.method, opts.precision, opts.tol, opts.maxit, opts.delta, 0, opts.check_every, 1,
                  opts.use_graph, opts.ell)
    solve!(λ, A, g; opts=o)
    return λ
end

# Replace the diagonal of ε: ε_cc at every E_c sample (3·Ncell reals in the DOF
# order c + 3·cell); the off-diagonal terms stay as they are.
function set_eps_diag!(A::FDFDOperator, ε::Vector{Float64})
    length(ε) == A.n || throw(DimensionMismatch("ε needs one value per E sample"))
    off = zeros(Float64, A.n)   # ε_xy, ε_yz, ε_zx at each cell's corner, read back and passed on unchanged
    check(ccall((:fdfd_get_eps, libfdfd), Cint, (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Ptr{UInt8}),
                A.h, C_NULL, off, C_NULL), A.h)
    check(ccall((:fdfd_set_eps, libfdfd), Cint, (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}), A.h, ε, off), A.h)
    return A
end

# e = A(ε) \ b with the diagonal ε given per E sample: the differentiable form
# of the solve (ε enters A = Cₘ Cₑ − ω² Pε, src/model/model.jl:235-237).
function solve_with_eps(A::FDFDOperator, ε::Vector{Float64}, b::Vector{ComplexF64}; opts::SolveOpts=SolveOpts())
    set_eps_diag!(A, ε)
    return first(solve!(zeros(ComplexF64, length(b)), A, b; opts=opts))
end

# Reverse rule of solve_with_eps, in ChainRulesCore's convention for complex
# values (a cotangent ē satisfies dL = Re(ēᴴ de)).  With g = conj(ē)/2 the
# Wirtinger derivative and transpose(A) λ = g solved on the GPU:
#   ∂A/∂ε_cc = −ω² on the diagonal  ⇒  ε̄_cc = 2Re(ω² λ_c e_c),
#   e = A⁻¹ b                      ⇒  b̄ = 2 conj(λ).
function ChainRulesCore.rrule(::typeof(solve_with_eps), A::FDFDOperator, ε::Vector{Float64},
                              b::Vector{ComplexF64}; opts::SolveOpts=SolveOpts())
    e = solve_with_eps(A, ε, b; opts=opts)
    function solve_with_eps_pullback(ē)
        g = conj.(unthunk(ē)) ./ 2
        λ = solve_pullback(A, e, g; opts=opts)
        ε̄ = 2 .* real.((A.ω^2) .* λ .* e)
        b̄ = 2 .* conj.(λ)
        return NoTangent(), NoTangent(), ε̄, b̄
    end
    return e, solve_with_eps_pullback
end

# Reverse rule of A \ b with respect to b (A held fixed): b̄ = 2 conj(λ).
function ChainRulesCore.rrule(::typeof(\), A::FDFDOperator, b::Vector{ComplexF64})
    e = A \ b
    function ldiv_pullback(ē)
        λ = solve_pullback(A, e, conj.(unthunk(ē)) ./ 2)
        return NoTangent(), NoTangent(), 2 .* conj.(λ)
    end
    return e, ldiv_pullback
end

# True residual r = b − A x and ‖r‖² on device buffers (CUDA.jl CuArray
# pointers, interleaved complex128): fdfd_residual_dev grows the handle's
# reduction buffer on first use; fdfd_residual_dev_noalloc allocates nothing
# (its scratch is a fixed static device array; E formulation only, grids up
# to 16384 x-y tiles of 32×8 cells).  Both return after ‖r‖² is on the host.
function residual_dev!(A::FDFDOperator, r::Ptr{Cvoid}, x::Ptr{Cvoid}, b::Ptr{Cvoid})
    nrm2 = Ref{Float64}(0.0)
    check(ccall((:fdfd_residual_dev, libfdfd), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ref{Float64}),
                A.h, x, b, r, nrm2), A.h)
    return nrm2[]
end
function residual_dev_noalloc!(A::FDFDOperator, r::Ptr{Cvoid}, x::Ptr{Cvoid}, b::Ptr{Cvoid})
    nrm2 = Ref{Float64}(0.0)
    check(ccall((:fdfd_residual_dev_noalloc, libfdfd), Cint,
                (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ref{Float64}), A.h, x, b, r, nrm2), A.h)
    return nrm2[]
end

# dL/dε_cc = 2Re(ω²λ_c e_c) at every E_c sample, as a (3, Nx, Ny, Nz) array
# (component fastest, the DOF order): one transposed solve on the GPU.
function eps_grad(A::FDFDOperator, e::Vector{ComplexF64}, g::Vector{ComplexF64}; opts::SolveOpts=SolveOpts())
    grad = zeros(Float64, length(e))
    st = Ref{SolveStats}()
    check(ccall((:fdfd_eps_grad, libfdfd), Cint,
                (Ptr{Cvoid}, Ptr{ComplexF64}, Ptr{ComplexF64}, Ptr{Float64}, Ref{SolveOpts}, Ref{SolveStats}),
                A.h, e, g, grad, opts, st), A.h)
    return grad, st[]
end

# H = (i/ω)(Cₑe + jₘ) — MaxwellFDFD.h_from_e(e, ω, (Pε,Pμ), (Cₑ,Cₘ), (jₑ,jₘ)) with Pμ = I.
function h_from_e(A::FDFDOperator, e::Vector{ComplexF64}, jₘ::Union{Nothing,Vector{ComplexF64}}=nothing)
    h = similar(e)
    check(ccall((:fdfd_h_from_e, libfdfd), Cint, (Ptr{Cvoid}, Ptr{ComplexF64}, Ptr{ComplexF64}, Ptr{ComplexF64}),
                A.h, e, jₘ === nothing ? C_NULL : jₘ, h), A.h)
    return h
end

# E = (−i/ω)Pε⁻¹(Cₘh − jₑ) — MaxwellFDFD.e_from_h(h, ω, (Pε,Pμ), (Cₑ,Cₘ), (jₑ,jₘ)) for a diagonal Pε.
function e_from_h(A::FDFDOperator, h::Vector{ComplexF64}, jₑ::Union{Nothing,Vector{ComplexF64}}=nothing)
    e = similar(h)
    check(ccall((:fdfd_e_from_h, libfdfd), Cint, (Ptr{Cvoid}, Ptr{ComplexF64}, Ptr{ComplexF64}, Ptr{ComplexF64}),
                A.h, h, jₑ === nothing ? C_NULL : jₑ, e), A.h)
    return e
end

# Mcₑ*e and Mcₘ*h of MaxwellFDFD.create_Mcs(mdl): fields at the voxel corners.
function corner_mean(A::FDFDOperator, v::Vector{ComplexF64}; field::Symbol=:E)
    out = similar(v)
    check(ccall((:fdfd_corner_mean, libfdfd), Cint, (Ptr{Cvoid}, Int32, Ptr{ComplexF64}, Ptr{ComplexF64}),
                A.h, field === :E ? 0 : 1, v, out), A.h)
    return out
end

end # module
