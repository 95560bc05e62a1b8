# MaxwellFDFDGPU — ccall binding of libfdfd_gb300 for MaxwellFDFD.jl.
#
# A GPU operator type that is a drop-in for the SparseMatrixCSC that
# MaxwellFDFD.create_A returns (src/model/model.jl:238-259): it implements
# size, eltype, mul!, *, transpose-mul, ldiv!/\ (GPU Krylov solve) and an
# rrule for the solve.  Signatures mirror include/fdfd_gb300.h one for one.
module MaxwellFDFDGPU

using LinearAlgebra
using MaxwellFDFD

export FDFDOperator, create_A_gpu, SolveOpts, eps_grad, h_from_e, e_from_h, corner_mean

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
    A = FDFDOperator(h[], 3prod(N), N)
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
# derivative, dL = 2Re(gᵀde)), λ solves transpose(A) λ = g and ∂L/∂b = λ;
# ∂L/∂A enters through ε (eps_grad below).  Written against ChainRulesCore
# when it is loaded.
function solve_pullback(A::FDFDOperator, e::Vector{ComplexF64}, g::Vector{ComplexF64}; opts::SolveOpts=SolveOpts())
    λ = zeros(ComplexF64, length(g))
    o = SolveOpts(opts.method, opts.precision, opts.tol, opts.maxit, opts.delta, 0, opts.check_every, 1,
                  opts.use_graph, opts.ell)
    solve!(λ, A, g; opts=o)
    return λ
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
