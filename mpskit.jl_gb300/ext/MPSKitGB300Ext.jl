# Package extension a maintainer adds next to ext/MPSKitAdaptExt.jl to route MPSKit's
# derivative operators, their Krylov solves and the environment transfers to libmpsgb.so
# (the C ABI of include/mpsgb.h).  Project.toml entries:
#
#   [weakdeps]   MPSKitGB300 = "<uuid of a tiny package that ships libmpsgb.so>"
#   [extensions] MPSKitGB300Ext = "MPSKitGB300"
#
# User code stays a drop-in:
#   find_groundstate(ψ, H, DMRG2(; trunc = truncrank(2048), backend = GB300Backend(:bf16x3)))
module MPSKitGB300Ext

using MPSKit
using MPSKit: JordanMPOTensor, MPOHamiltonian, DerivativeOperator
using TensorKit
using TensorOperations: AbstractBackend
using KrylovKit: Lanczos
import MPSKit: AC_hamiltonian, AC2_hamiltonian, C_hamiltonian, fixedpoint

const libmpsgb = get(ENV, "MPSGB_LIB", "libmpsgb.so")

const GB_OK = Cint(0)
const GB_F64, GB_C128 = Cint(1), Cint(2)
const GB_KIND_MPS, GB_KIND_BOND, GB_KIND_AC2 = Cint(1), Cint(2), Cint(3)
const GB_KIND_GL, GB_KIND_GR, GB_KIND_MPO = Cint(4), Cint(5), Cint(6)
const GB_HEFF_C, GB_HEFF_AC, GB_HEFF_AC2 = Cint(0), Cint(1), Cint(2)

struct KrylovInfoC
    converged::Cint
    numops::Cint
    numiter::Cint
    normres::Cdouble
end

"""
    GB300Backend(precision = :fp64; device = 0)

`TensorOperations.AbstractBackend` selecting the GB300 engine.  `precision` is `:fp64`
(plain), `:bf16x3` or `:tf32x3` (split-precision tensor-core contractions with BF16 or TF32
hi/lo operands, FP64 Krylov and gauge).
"""
struct GB300Backend <: AbstractBackend
    precision::Cint
    device::Cint
end
const PRECISION_CODES = Dict(:fp64 => Cint(0), :bf16x3 => Cint(1), :tf32x3 => Cint(2))
GB300Backend(p::Symbol = :fp64; device::Integer = 0) =
    GB300Backend(PRECISION_CODES[p], Cint(device))

check(code) = code == GB_OK ? nothing :
    error("libmpsgb: ", unsafe_string(ccall((:gb_last_error, libmpsgb), Cstring, ())))

# one context per (task, device), as the C ABI requires for concurrent callers
const CTX = Dict{Tuple{UInt, Cint}, Ptr{Cvoid}}()
function context(dev::Cint)
    key = (objectid(current_task()), dev)
    get!(CTX, key) do
        r = Ref{Ptr{Cvoid}}()
        check(ccall((:gb_ctx_create, libmpsgb), Cint, (Cint, UInt32, Ptr{Ptr{Cvoid}}), dev, 0, r))
        r[]
    end
end

dtype(T) = T <: Complex ? GB_C128 : GB_F64

"""Upload the dense block of a Trivial-sector TensorMap (or a dense JordanMPOTensor)."""
function upload(ctx, kind::Cint, t::AbstractArray{T}) where {T}
    dims = Int64[size(t)...]
    r = Ref{Ptr{Cvoid}}()
    check(ccall((:gb_tensor_create, libmpsgb), Cint,
                (Ptr{Cvoid}, Cint, Cint, Cint, Ptr{Int64}, Ptr{Ptr{Cvoid}}),
                ctx, kind, dtype(T), length(dims), dims, r))
    check(ccall((:gb_tensor_upload, libmpsgb), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Csize_t),
                r[], t, sizeof(t)))
    return r[]
end
function download!(t::AbstractArray, h::Ptr{Cvoid})
    check(ccall((:gb_tensor_download, libmpsgb), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Csize_t),
                h, t, sizeof(t)))
    return t
end
free(h) = ccall((:gb_tensor_free, libmpsgb), Cint, (Ptr{Cvoid},), h)

# dense channel-sum-space array of a JordanMPOTensor: W[wl, s, s', wr]
densempo(W::JordanMPOTensor) = convert(Array, TensorMap(W))
denseenv(G) = convert(Array, G isa TensorMap ? G : TensorMap(G))

# Symmetric tensors cross the boundary as their dense embedding.  For U1Irrep spaces
# TensorKit iterates the sectors of a leg in sorted charge order, so convert(Array, t) is
# the charge-sorted layout libmpsgb's U(1) path expects (zeros outside the blocks); the
# way back is the projecting constructor TensorMap(array, space).
fromdense(a::AbstractArray, V) = TensorMap(a, V)
# per-index charges of a U1 leg (2q, so spin-1/2 charges are odd integers), as the
# gb_u1_* factorisations take them
leg_charges(V) = Int32[Int32(2 * c.charge) for c in sectors(V) for _ in 1:dim(V, c)]

"""
    GB300Derivative <: DerivativeOperator

Handle of a prepared effective operator living on the GPU (gb_heff_build); applying it or
calling `fixedpoint` on it runs on the device.
"""
mutable struct GB300Derivative{T, N} <: DerivativeOperator
    h::Ptr{Cvoid}
    ctx::Ptr{Cvoid}
    kind::Cint
    xspace::Any              # TensorMapSpace of the vectors it acts on
    keep::Vector{Ptr{Cvoid}} # device tensors referenced by the operator
end

function build(kind, ctx, GL, Ws, GR, xspace, T, backend::GB300Backend)
    hGL = upload(ctx, GB_KIND_GL, denseenv(GL))
    hGR = upload(ctx, GB_KIND_GR, denseenv(GR))
    hW = [upload(ctx, GB_KIND_MPO, densempo(W)) for W in Ws]
    r = Ref{Ptr{Cvoid}}()
    w1 = length(hW) ≥ 1 ? hW[1] : C_NULL
    w2 = length(hW) ≥ 2 ? hW[2] : C_NULL
    check(ccall((:gb_heff_build, libmpsgb), Cint,
                (Ptr{Cvoid}, Cint, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Cint,
                 Ptr{Ptr{Cvoid}}), ctx, kind, hGL, w1, w2, hGR, backend.precision, r))
    N = kind == GB_HEFF_AC2 ? 4 : kind == GB_HEFF_AC ? 3 : 2
    if kind != GB_HEFF_C && sectortype(xspace) === U1Irrep
        # the vectors' U(1) sectors: x[l s1; r s2] allowed where q_l + q_s1 + q_s2 = q_r
        ql, qs1 = leg_charges(codomain(xspace)[1]), leg_charges(codomain(xspace)[2])
        qr = leg_charges(domain(xspace)[1])
        qs2 = kind == GB_HEFF_AC2 ? leg_charges(dual(domain(xspace)[2])) : C_NULL
        check(ccall((:gb_heff_set_sectors, libmpsgb), Cint,
                    (Ptr{Cvoid}, Ptr{Int32}, Ptr{Int32}, Ptr{Int32}, Ptr{Int32}),
                    r[], ql, qs1, qs2, qr))
    end
    op = GB300Derivative{T, N}(r[], ctx, kind, xspace, [hGL; hGR; hW])
    finalizer(op) do o
        ccall((:gb_heff_free, libmpsgb), Cint, (Ptr{Cvoid},), o.h)
        foreach(free, o.keep)
    end
    return op
end

xkind(op) = op.kind == GB_HEFF_AC2 ? GB_KIND_AC2 : op.kind == GB_HEFF_AC ? GB_KIND_MPS : GB_KIND_BOND

# hamiltonian_derivatives.jl:44-55
function AC_hamiltonian(site::Int, below, operator::MPOHamiltonian, above, envs;
                        backend::GB300Backend, kwargs...)
    ctx = context(backend.device)
    GL, GR = leftenv(envs, site, below), rightenv(envs, site, below)
    T = scalartype(GL)
    return build(GB_HEFF_AC, ctx, GL, (operator[site],), GR, space(below.AC[site]), T, backend)
end
# hamiltonian_derivatives.jl:206-217
function AC2_hamiltonian(site::Int, below, operator::MPOHamiltonian, above, envs;
                         backend::GB300Backend, kwargs...)
    ctx = context(backend.device)
    GL, GR = leftenv(envs, site, below), rightenv(envs, site + 1, below)
    T = scalartype(GL)
    return build(GB_HEFF_AC2, ctx, GL, (operator[site], operator[site + 1]), GR,
                 space(AC2(below, site)), T, backend)
end
# mpo_derivatives.jl:37-45
function C_hamiltonian(site::Int, below, operator, above, envs; backend::GB300Backend, kwargs...)
    ctx = context(backend.device)
    GL, GR = leftenv(envs, site + 1, below), rightenv(envs, site, below)
    return build(GB_HEFF_C, ctx, GL, (), GR, space(below.C[site]), scalartype(GL), backend)
end

# (H)(x): upload, apply, download (derivatives.jl:10-11)
function (op::GB300Derivative{T})(x::AbstractTensorMap) where {T}
    hx = upload(op.ctx, xkind(op), convert(Array, x))
    hy = upload(op.ctx, xkind(op), zeros(T, size(convert(Array, x))))
    check(ccall((:gb_heff_apply, libmpsgb), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}),
                op.h, hx, hy))
    a = zeros(T, size(convert(Array, x)))
    download!(a, hy)
    free(hx); free(hy)
    return fromdense(a, space(x))
end

# fixedpoint.jl:15-18: the whole Lanczos eigensolve on the device
function fixedpoint(op::GB300Derivative{T}, x₀, which::Symbol, alg::Lanczos) where {T}
    which === :SR || throw(ArgumentError("only :SR runs on the device"))
    a = convert(Array, x₀)
    hx = upload(op.ctx, xkind(op), a)
    λ = Ref{Cdouble}()
    info = Ref{KrylovInfoC}()
    check(ccall((:gb_heff_eigsolve, libmpsgb), Cint,
                (Ptr{Cvoid}, Ptr{Cvoid}, Cint, Cint, Cdouble, Cint, Ptr{Cdouble},
                 Ptr{KrylovInfoC}), op.h, hx, alg.krylovdim, alg.maxiter, alg.tol, alg.eager,
                λ, info))
    download!(a, hx)
    free(hx)
    x = fromdense(a, space(x₀))
    i = info[]
    return λ[], x, (; converged = i.converged, numops = i.numops, numiter = i.numiter,
                    normres = (i.normres,))
end

end # module
