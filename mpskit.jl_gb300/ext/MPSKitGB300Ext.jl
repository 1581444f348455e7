# Package extension a maintainer adds next to ext/MPSKitAdaptExt.jl to route MPSKit's
# derivative operators, their Krylov solves, the truncated-SVD gauge step and the
# environment recursions to libmpsgb.so (the C ABI of include/mpsgb.h).  Project.toml:
#
#   [weakdeps]   MPSKitGB300 = "<uuid of a tiny package that ships libmpsgb.so>"
#   [extensions] MPSKitGB300Ext = "MPSKitGB300"
#
# User code stays a drop-in:
#   find_groundstate(ψ, H, DMRG2(; trunc = truncrank(2048) & trunctol(; atol = 1e-10),
#                                 backend = GB300Backend(:bf16x3)))
#
# Dispatch.  Every method below is strictly more specific, in its POSITIONAL arguments, than
# the reference method it takes over (a keyword never selects a method in Julia), and hands
# any backend other than GB300Backend back to that reference method with `invoke`:
#
#   AC_hamiltonian(::Int, ::FiniteMPS{<:MPSTensor}, ::FiniteMPOHamiltonian,
#                  ::FiniteMPS{<:MPSTensor}, ::FiniteEnvironments)
#       over  (::Int, ::_HAM_MPS_TYPES, ::MPOHamiltonian, ::_HAM_MPS_TYPES, envs)
#             src/algorithms/derivatives/hamiltonian_derivatives.jl:44-55
#   AC2_hamiltonian(same types)        over hamiltonian_derivatives.jl:206-217
#   C_hamiltonian(same types)          over (::Int, below, operator, above, envs)
#                                           src/algorithms/derivatives/mpo_derivatives.jl:37-45
#   (the InfiniteMPS / InfiniteMPOHamiltonian / InfiniteEnvironments variants likewise)
#   find_groundstate!(::FiniteMPS{<:MPSTensor}, ::FiniteMPOHamiltonian,
#                     ::DMRG2{<:Any, <:Any, <:Any, <:GB300Backend}, envs)
#       over  (::AbstractFiniteMPS, H, ::Union{DMRG, DMRG2}, envs)
#             src/algorithms/groundstate/dmrg.jl:279-285
#   fixedpoint(::GB300Derivative, x₀, ::Symbol, ::Lanczos)
#       over  (A, x₀, which::Symbol, alg::Lanczos)   src/algorithms/fixedpoint.jl:15-18
#
# Storage (the "device residency" seam): environments are uploaded once per host object --
# a cache keyed by the identity of the environment's storage array, the same `===`
# invalidation FiniteEnvironments uses (src/environments/finite_envs.jl:110-151) -- so a
# local update uploads only its start vector.  The DMRG2 overload keeps the whole sweep on
# the device (environments built there with gb_env_transfer_left/right, gauge2! through
# gb_svd_trunc / gb_u1_svd_trunc) and writes the state back once at the end.
#
# This file cannot run in the build container (no Julia there); the same C-ABI sequence is
# exercised on the GPU by the Python mirror (mpsgb.algorithms._sweep_dmrg2).
module MPSKitGB300Ext

using MPSKit
using MPSKit: DerivativeOperator, MPOHamiltonian, FiniteMPOHamiltonian, InfiniteMPOHamiltonian,
              FiniteEnvironments, InfiniteEnvironments, MPSTensor, DMRG2, AbstractFiniteMPS,
              _HAM_MPS_TYPES, adapt_solver, leftenv, rightenv
using TensorKit
using TensorOperations: AbstractBackend
using KrylovKit: Lanczos
import MPSKit: AC_hamiltonian, AC2_hamiltonian, C_hamiltonian, fixedpoint, find_groundstate!

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

# One context per (task, device), as the C ABI requires for concurrent callers; the table is
# shared by all tasks, so every access holds the lock.
const CTX_LOCK = ReentrantLock()
const CTX = Dict{Tuple{UInt, Cint}, Ptr{Cvoid}}()
function context(dev::Cint)
    key = (objectid(current_task()), dev)
    return lock(CTX_LOCK) do
        get!(CTX, key) do
            r = Ref{Ptr{Cvoid}}()
            check(ccall((:gb_ctx_create, libmpsgb), Cint, (Cint, UInt32, Ptr{Ptr{Cvoid}}),
                        dev, 0, r))
            r[]
        end
    end
end

dtype(T) = T <: Complex ? GB_C128 : GB_F64

"""Device tensor handle (freed by its finalizer)."""
mutable struct DTensor
    h::Ptr{Cvoid}
    dims::Vector{Int64}
    function DTensor(h::Ptr{Cvoid}, dims)
        t = new(h, Int64[dims...])
        finalizer(x -> ccall((:gb_tensor_free, libmpsgb), Cint, (Ptr{Cvoid},), x.h), t)
        return t
    end
end

function create(ctx, kind::Cint, T, dims)
    d = Int64[dims...]
    r = Ref{Ptr{Cvoid}}()
    check(ccall((:gb_tensor_create, libmpsgb), Cint,
                (Ptr{Cvoid}, Cint, Cint, Cint, Ptr{Int64}, Ptr{Ptr{Cvoid}}),
                ctx, kind, dtype(T), length(d), d, r))
    return DTensor(r[], d)
end
"""Upload the dense block of a TensorMap (for U1Irrep legs: the charge-sorted embedding)."""
function upload(ctx, kind::Cint, a::AbstractArray{T}) where {T}
    t = create(ctx, kind, T, size(a))
    check(ccall((:gb_tensor_upload, libmpsgb), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Csize_t),
                t.h, a, sizeof(a)))
    return t
end
function download(t::DTensor, ::Type{T}) where {T}
    a = zeros(T, Tuple(t.dims))
    check(ccall((:gb_tensor_download, libmpsgb), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Csize_t),
                t.h, a, sizeof(a)))
    return a
end
function wrap(h::Ptr{Cvoid})
    kind, dt, nd = Ref{Cint}(), Ref{Cint}(), Ref{Cint}()
    dims = zeros(Int64, 6)
    check(ccall((:gb_tensor_shape, libmpsgb), Cint,
                (Ptr{Cvoid}, Ptr{Cint}, Ptr{Cint}, Ptr{Cint}, Ptr{Int64}), h, kind, dt, nd, dims))
    return DTensor(h, dims[1:nd[]])
end

# dense channel-sum-space array of a JordanMPOTensor: W[wl, s, s', wr]
densempo(W) = convert(Array, TensorMap(W))
denseenv(G) = convert(Array, G isa TensorMap ? G : TensorMap(G))
fromdense(a::AbstractArray, V) = TensorMap(a, V)

# per-index charges of a U1 leg (2q, so spin-1/2 charges are odd integers); TensorKit lists
# the sectors of a graded space in ascending order, the layout of the charge-sorted embedding
leg_charges(V) = Int32[Int32(2 * c.charge) for c in sectors(V) for _ in 1:dim(V, c)]
isu1(V) = sectortype(V) === U1Irrep

# Environments on the device, uploaded once per host environment object: keyed by the
# identity of its storage array (a new environment is a new array), released with it.
const ENV_LOCK = ReentrantLock()
const ENV_CACHE = WeakKeyDict{Any, DTensor}()
storage(G) = G isa TensorMap ? G.data : G
function device_env(ctx, kind::Cint, G)
    key = storage(G)
    return lock(ENV_LOCK) do
        get!(ENV_CACHE, key) do
            upload(ctx, kind, denseenv(G))
        end
    end
end

"""
    GB300Derivative <: DerivativeOperator

Handle of a prepared effective operator living on the GPU (gb_heff_build); applying it or
calling `fixedpoint` on it runs on the device.
"""
mutable struct GB300Derivative{T, N} <: DerivativeOperator
    h::Ptr{Cvoid}
    ctx::Ptr{Cvoid}
    kind::Cint
    xspace::Any          # TensorMapSpace of the vectors it acts on
    keep::Vector{Any}    # device tensors referenced by the operator
end

function set_sectors!(h, kind, xspace)
    (kind == GB_HEFF_C || !isu1(xspace)) && return nothing
    # x[l s1; r s2] allowed where q_l + q_s1 + q_s2 = q_r (one-site: q_l + q_s = q_r)
    ql, qs1 = leg_charges(codomain(xspace)[1]), leg_charges(codomain(xspace)[2])
    qr = leg_charges(domain(xspace)[1])
    qs2 = kind == GB_HEFF_AC2 ? leg_charges(dual(domain(xspace)[2])) : C_NULL
    check(ccall((:gb_heff_set_sectors, libmpsgb), Cint,
                (Ptr{Cvoid}, Ptr{Int32}, Ptr{Int32}, Ptr{Int32}, Ptr{Int32}), h, ql, qs1, qs2, qr))
    return nothing
end

function build(kind, ctx, dGL::DTensor, dWs, dGR::DTensor, xspace, T, backend::GB300Backend)
    r = Ref{Ptr{Cvoid}}()
    w1 = length(dWs) ≥ 1 ? dWs[1].h : C_NULL
    w2 = length(dWs) ≥ 2 ? dWs[2].h : C_NULL
    check(ccall((:gb_heff_build, libmpsgb), Cint,
                (Ptr{Cvoid}, Cint, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Cint,
                 Ptr{Ptr{Cvoid}}), ctx, kind, dGL.h, w1, w2, dGR.h, backend.precision, r))
    set_sectors!(r[], kind, xspace)
    N = kind == GB_HEFF_AC2 ? 4 : kind == GB_HEFF_AC ? 3 : 2
    op = GB300Derivative{T, N}(r[], ctx, kind, xspace, Any[dGL, dGR, dWs...])
    finalizer(o -> ccall((:gb_heff_free, libmpsgb), Cint, (Ptr{Cvoid},), o.h), op)
    return op
end

# the MPO tensors of a Hamiltonian on the device, once per (Hamiltonian, context)
const MPO_LOCK = ReentrantLock()
const MPO_CACHE = WeakKeyDict{Any, Dict{Ptr{Cvoid}, Vector{DTensor}}}()
function device_mpo(ctx, H)
    return lock(MPO_LOCK) do
        byctx = get!(() -> Dict{Ptr{Cvoid}, Vector{DTensor}}(), MPO_CACHE, H)
        get!(byctx, ctx) do
            [upload(ctx, GB_KIND_MPO, densempo(H[i])) for i in 1:length(H)]
        end
    end
end

xkind(op) = op.kind == GB_HEFF_AC2 ? GB_KIND_AC2 : op.kind == GB_HEFF_AC ? GB_KIND_MPS : GB_KIND_BOND

# ---------------------------------------------------------------- derivative constructors
const _FIN = FiniteMPS{<:MPSTensor}
const _INF = InfiniteMPS{<:MPSTensor}

for (MPS, HAM, ENV) in ((_FIN, FiniteMPOHamiltonian, FiniteEnvironments),
                        (_INF, InfiniteMPOHamiltonian, InfiniteEnvironments))
    @eval begin
        # hamiltonian_derivatives.jl:44-55
        function AC_hamiltonian(site::Int, below::$MPS, operator::$HAM, above::$MPS, envs::$ENV;
                                backend::AbstractBackend = MPSKit.Defaults.backend(), kwargs...)
            backend isa GB300Backend ||
                return invoke(AC_hamiltonian,
                              Tuple{Int, _HAM_MPS_TYPES, MPOHamiltonian, _HAM_MPS_TYPES, Any},
                              site, below, operator, above, envs; backend, kwargs...)
            ctx = context(backend.device)
            GL, GR = leftenv(envs, site, below), rightenv(envs, site, below)
            W = device_mpo(ctx, operator)
            return build(GB_HEFF_AC, ctx, device_env(ctx, GB_KIND_GL, GL), (W[site],),
                         device_env(ctx, GB_KIND_GR, GR), space(below.AC[site]), scalartype(GL),
                         backend)
        end
        # hamiltonian_derivatives.jl:206-217
        function AC2_hamiltonian(site::Int, below::$MPS, operator::$HAM, above::$MPS, envs::$ENV;
                                 backend::AbstractBackend = MPSKit.Defaults.backend(), kwargs...)
            backend isa GB300Backend ||
                return invoke(AC2_hamiltonian,
                              Tuple{Int, _HAM_MPS_TYPES, MPOHamiltonian, _HAM_MPS_TYPES, Any},
                              site, below, operator, above, envs; backend, kwargs...)
            ctx = context(backend.device)
            GL, GR = leftenv(envs, site, below), rightenv(envs, site + 1, below)
            W = device_mpo(ctx, operator)
            return build(GB_HEFF_AC2, ctx, device_env(ctx, GB_KIND_GL, GL), (W[site], W[site + 1]),
                         device_env(ctx, GB_KIND_GR, GR), space(MPSKit.AC2(below, site)),
                         scalartype(GL), backend)
        end
        # mpo_derivatives.jl:37-45
        function C_hamiltonian(site::Int, below::$MPS, operator::$HAM, above::$MPS, envs::$ENV;
                               backend::AbstractBackend = MPSKit.Defaults.backend(), kwargs...)
            backend isa GB300Backend ||
                return invoke(C_hamiltonian, Tuple{Int, Any, Any, Any, Any},
                              site, below, operator, above, envs; backend, kwargs...)
            ctx = context(backend.device)
            GL, GR = leftenv(envs, site + 1, below), rightenv(envs, site, below)
            return build(GB_HEFF_C, ctx, device_env(ctx, GB_KIND_GL, GL), (),
                         device_env(ctx, GB_KIND_GR, GR), space(below.C[site]), scalartype(GL),
                         backend)
        end
    end
end

# (H)(x): upload, apply, download (derivatives.jl:10-11)
function (op::GB300Derivative{T})(x::AbstractTensorMap) where {T}
    a = convert(Array, x)
    hx = upload(op.ctx, xkind(op), a)
    hy = create(op.ctx, xkind(op), T, size(a))
    check(ccall((:gb_heff_apply, libmpsgb), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}),
                op.h, hx.h, hy.h))
    return fromdense(download(hy, T), space(x))
end

# fixedpoint.jl:15-18: the whole Lanczos eigensolve on the device
function fixedpoint(op::GB300Derivative{T}, x₀, which::Symbol, alg::Lanczos) where {T}
    which === :SR || throw(ArgumentError("only :SR runs on the device"))
    hx = upload(op.ctx, xkind(op), convert(Array, x₀))
    λ = Ref{Cdouble}()
    info = Ref{KrylovInfoC}()
    check(ccall((:gb_heff_eigsolve, libmpsgb), Cint,
                (Ptr{Cvoid}, Ptr{Cvoid}, Cint, Cint, Cdouble, Cint, Ptr{Cdouble},
                 Ptr{KrylovInfoC}), op.h, hx.h, alg.krylovdim, alg.maxiter, alg.tol, alg.eager,
                λ, info))
    x = fromdense(download(hx, T), space(x₀))
    i = info[]
    return λ[], x, (; converged = i.converged, numops = i.numops, numiter = i.numiter,
                    normres = (i.normres,))
end

# ---------------------------------------------------------------- DMRG2 on the device
# truncrank(n) & trunctol(; atol) of the TruncatedAlgorithm carried by DMRG2.alg_gauge
function trunc_params(strategy)
    maxdim, atol = 0, 0.0
    walk(t) = if hasproperty(t, :components)
        foreach(walk, t.components)
    else
        hasproperty(t, :howmany) && (maxdim = Int(t.howmany))
        hasproperty(t, :atol) && (atol = Float64(t.atol))
    end
    walk(strategy)
    return maxdim, atol
end

"""Device-resident copy of a FiniteMPS: AL/AR/C handles, the centre bond and, for U(1)
states, the charges of every bond."""
mutable struct DeviceMPS
    AL::Vector{Union{Nothing, DTensor}}
    AR::Vector{Union{Nothing, DTensor}}
    C::Vector{Union{Nothing, DTensor}}
    qb::Union{Nothing, Vector{Vector{Int32}}}
    qp::Union{Nothing, Vector{Int32}}
    ctx::Ptr{Cvoid}
end

function ac2(ctx, A::DTensor, B::DTensor, T)
    out = create(ctx, GB_KIND_AC2, T, (A.dims[1], A.dims[2], B.dims[3], B.dims[2]))
    check(ccall((:gb_mps_ac2, libmpsgb), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}),
                ctx, A.h, B.h, out.h))
    return out
end
function mul(ctx, f::Symbol, X::DTensor, Y::DTensor, dims, T)
    out = create(ctx, GB_KIND_MPS, T, dims)
    check(ccall((f, libmpsgb), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}),
                ctx, X.h, Y.h, out.h))
    return out
end
function env_step(ctx, side, G::DTensor, W::DTensor, A::DTensor, prec, T)
    if side === :left
        out = create(ctx, GB_KIND_GL, T, (A.dims[3], W.dims[4], A.dims[3]))
        check(ccall((:gb_env_transfer_left, libmpsgb), Cint,
                    (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Cint, Ptr{Cvoid}),
                    ctx, G.h, W.h, A.h, A.h, prec, out.h))
    else
        out = create(ctx, GB_KIND_GR, T, (A.dims[1], W.dims[1], A.dims[1]))
        check(ccall((:gb_env_transfer_right, libmpsgb), Cint,
                    (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Cint, Ptr{Cvoid}),
                    ctx, G.h, W.h, A.h, A.h, prec, out.h))
    end
    return out
end

# gauge2! (src/states/orthoview.jl:401-420) on the device; returns AL, C, AR and eps
function svd_trunc(ctx, x::DTensor, maxdim, atol, st::DeviceMPS, pos)
    a, s, r, eps = Ref{Ptr{Cvoid}}(), Ref{Ptr{Cvoid}}(), Ref{Ptr{Cvoid}}(), Ref{Cdouble}()
    if st.qb === nothing
        check(ccall((:gb_svd_trunc, libmpsgb), Cint,
                    (Ptr{Cvoid}, Ptr{Cvoid}, Int64, Cdouble, Cint, Ptr{Ptr{Cvoid}},
                     Ptr{Ptr{Cvoid}}, Ptr{Ptr{Cvoid}}, Ptr{Cdouble}),
                    ctx, x.h, maxdim, atol, 1, a, s, r, eps))
    else
        qk = zeros(Int32, min(x.dims[1] * x.dims[2], x.dims[3] * x.dims[4]))
        k = Ref{Int64}()
        check(ccall((:gb_u1_svd_trunc, libmpsgb), Cint,
                    (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Int32}, Ptr{Int32}, Ptr{Int32}, Ptr{Int32}, Int64,
                     Cdouble, Cint, Ptr{Ptr{Cvoid}}, Ptr{Ptr{Cvoid}}, Ptr{Ptr{Cvoid}}, Ptr{Int32},
                     Ptr{Int64}, Ptr{Cdouble}),
                    ctx, x.h, st.qb[pos], st.qp, st.qb[pos + 2], st.qp, maxdim, atol, 1, a, s, r,
                    qk, k, eps))
        st.qb[pos + 1] = qk[1:k[]]
    end
    return wrap(a[]), wrap(s[]), wrap(r[]), eps[]
end

function operator_ac2(ctx, GL, W, GR, pos, x::DTensor, st::DeviceMPS, T, backend)
    r = Ref{Ptr{Cvoid}}()
    check(ccall((:gb_heff_build, libmpsgb), Cint,
                (Ptr{Cvoid}, Cint, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Cint,
                 Ptr{Ptr{Cvoid}}), ctx, GB_HEFF_AC2, GL.h, W[pos].h, W[pos + 1].h, GR.h,
                backend.precision, r))
    op = GB300Derivative{T, 4}(r[], ctx, GB_HEFF_AC2, nothing, Any[GL, GR])
    finalizer(o -> ccall((:gb_heff_free, libmpsgb), Cint, (Ptr{Cvoid},), o.h), op)
    if st.qb !== nothing
        check(ccall((:gb_heff_set_sectors, libmpsgb), Cint,
                    (Ptr{Cvoid}, Ptr{Int32}, Ptr{Int32}, Ptr{Int32}, Ptr{Int32}),
                    op.h, st.qb[pos], st.qp, st.qp, st.qb[pos + 2]))
    end
    return op
end

function eigsolve!(op, x::DTensor, alg)
    λ = Ref{Cdouble}()
    info = Ref{KrylovInfoC}()
    check(ccall((:gb_heff_eigsolve, libmpsgb), Cint,
                (Ptr{Cvoid}, Ptr{Cvoid}, Cint, Cint, Cdouble, Cint, Ptr{Cdouble},
                 Ptr{KrylovInfoC}), op.h, x.h, alg.krylovdim, alg.maxiter, alg.tol, alg.eager,
                λ, info))
    return λ[], info[]
end

"""
    find_groundstate!(ψ::FiniteMPS, H::FiniteMPOHamiltonian, alg::DMRG2 with GB300Backend)

The DMRG2 sweep of src/algorithms/groundstate/dmrg.jl:211-354 with every tensor on the
device: the state and the MPO are uploaded once; each bond update builds the operator
(gb_heff_build, the U(1) sectors passed along), runs the Galerkin matvec, the adaptive
Lanczos (adapt_solver of the algorithm's own AdaptiveKrylov) and the truncated SVD on the
device; environments are advanced on the device.  The converged state comes back as a new
FiniteMPS (the returned value; `find_groundstate` returns it as the reference does).
"""
function find_groundstate!(ψ::_FIN, H::FiniteMPOHamiltonian,
                           alg::DMRG2{<:Any, <:Any, <:Any, <:GB300Backend}, envs = nothing)
    T = scalartype(ψ)
    be = alg.backend
    ctx = context(be.device)
    n = length(ψ)
    maxdim, atol = trunc_params(alg.alg_gauge.trunc)
    W = device_mpo(ctx, H)
    u1 = isu1(space(ψ.AL[1]))
    qb = u1 ? [leg_charges(left_virtualspace(ψ, i)) for i in 1:n] : nothing
    u1 && push!(qb, leg_charges(right_virtualspace(ψ, n)))
    qp = u1 ? leg_charges(physicalspace(ψ, 1)) : nothing
    st = DeviceMPS(Vector{Union{Nothing, DTensor}}(nothing, n),
                   Vector{Union{Nothing, DTensor}}(nothing, n),
                   Vector{Union{Nothing, DTensor}}(nothing, n + 1), qb, qp, ctx)
    # right-canonical start: AC[1] = C[1] AR[1]
    for i in 1:n
        st.AR[i] = upload(ctx, GB_KIND_MPS, convert(Array, ψ.AR[i]))
    end
    st.C[1] = upload(ctx, GB_KIND_BOND, convert(Array, ψ.C[0]))
    GL = Vector{Union{Nothing, DTensor}}(nothing, n)
    GR = Vector{Union{Nothing, DTensor}}(nothing, n)
    GL[1] = upload(ctx, GB_KIND_GL, ones(T, 1, 1, 1))
    GR[n] = upload(ctx, GB_KIND_GR, ones(T, 1, 1, 1))
    for i in n:-1:2
        GR[i - 1] = env_step(ctx, :right, GR[i], W[i], st.AR[i], be.precision, T)
    end
    ϵ_locals, ϵ_truncs, decays = ones(n - 1), zeros(n - 1), zeros(n - 1)
    ϵ_global = 1.0
    center = 1          # AC of site `center` = C[center] AR[center]
    for iter in 1:(alg.maxiter)
        for (dir, range) in ((:right, 1:(n - 1)), (:left, (n - 2):-1:1))
            for pos in range
                # AC2 of sites (pos, pos + 1) from the current centre
                if dir === :right
                    # AC of site pos: C AR when the centre bond is left of it, AL C when right
                    acl = center == pos ?
                          mul(ctx, :gb_mps_mul_front, st.C[pos], st.AR[pos],
                              (st.C[pos].dims[1], st.AR[pos].dims[2], st.AR[pos].dims[3]), T) :
                          mul(ctx, :gb_mps_mul_tail, st.AL[pos], st.C[pos + 1],
                              (st.AL[pos].dims[1], st.AL[pos].dims[2], st.C[pos + 1].dims[2]), T)
                    # the left-gauged tensor of site pos for the Galerkin projector
                    center == pos && (st.AL[pos] = left_orth(ctx, acl))
                    x = ac2(ctx, acl, st.AR[pos + 1], T)
                else
                    acr = mul(ctx, :gb_mps_mul_tail, st.AL[pos + 1], st.C[pos + 2],
                              (st.AL[pos + 1].dims[1], st.AL[pos + 1].dims[2],
                               st.C[pos + 2].dims[2]), T)
                    x = ac2(ctx, st.AL[pos], acr, T)
                end
                op = operator_ac2(ctx, GL[pos], W, GR[pos + 1], pos, x, st, T, be)
                y = create(ctx, GB_KIND_AC2, T, x.dims)
                check(ccall((:gb_heff_apply, libmpsgb), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}),
                            op.h, x.h, y.h))
                ϵ_local = galerkin(ctx, y, st.AL[pos])
                solver = adapt_solver(alg.alg_eigsolve; decay_rate = decays[pos],
                                      g_local = ϵ_local, g_global = ϵ_global,
                                      eps_trunc = ϵ_truncs[pos])
                _, info = eigsolve!(op, x, solver)
                al, c, ar, ϵ_trunc = svd_trunc(ctx, x, maxdim, atol, st, pos)
                st.AL[pos], st.C[pos + 1], st.AR[pos + 1] = al, c, ar
                center = pos + 1
                dir === :right && (GL[pos + 1] = env_step(ctx, :left, GL[pos], W[pos], al,
                                                          be.precision, T))
                dir === :left && (GR[pos] = env_step(ctx, :right, GR[pos + 1], W[pos + 1], ar,
                                                     be.precision, T))
                ϵ_locals[pos], ϵ_truncs[pos] = ϵ_local, ϵ_trunc
                decays[pos] = clamp((info.normres / ϵ_local)^(1 / max(1, info.numops)),
                                    1.0e-3, 0.999)
                ϵ_global = maximum(ϵ_locals)
            end
        end
        ϵ_global = maximum(ϵ_locals)
        ϵ_global <= max(alg.tol, maximum(ϵ_truncs)) && break
    end
    ψ′ = writeback(ψ, st, T)
    return ψ′, MPSKit.environments(ψ′, H), ϵ_global
end

# |(1 - AL AL') normalize(H x)| (src/algorithms/groundstate/dmrg.jl:220-223)
function galerkin(ctx, y::DTensor, AL::DTensor)
    nrm = Ref{Cdouble}()
    check(ccall((:gb_tensor_norm, libmpsgb), Cint, (Ptr{Cvoid}, Ptr{Cdouble}), y.h, nrm))
    check(ccall((:gb_tensor_scale, libmpsgb), Cint, (Ptr{Cvoid}, Cdouble, Cdouble),
                y.h, 1 / nrm[], 0.0))
    check(ccall((:gb_project_complement, libmpsgb), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}),
                ctx, y.h, AL.h))
    check(ccall((:gb_tensor_norm, libmpsgb), Cint, (Ptr{Cvoid}, Ptr{Cdouble}), y.h, nrm))
    return nrm[]
end

# left_gauge(AC) with positive Householder QR (src/states/orthoview.jl:322-326); the U(1)
# variant is not needed here: the QR of a charge-conserving AC stays charge-conserving
function left_orth(ctx, AC::DTensor)
    q, r = Ref{Ptr{Cvoid}}(), Ref{Ptr{Cvoid}}()
    check(ccall((:gb_left_orth, libmpsgb), Cint,
                (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Ptr{Cvoid}}, Ptr{Ptr{Cvoid}}), ctx, AC.h, q, r))
    wrap(r[])  # freed with its handle
    return wrap(q[])
end

# The device state after a full sweep: AL[1] C[2] AR[2..n] (centre bond between sites 1 and
# 2), returned as a FiniteMPS built from its site tensors [AL[1] C, AR[2], ..., AR[n]] (the
# FiniteMPS constructor re-gauges them on the host; the state is the same).
function writeback(ψ, st::DeviceMPS, T)
    n = length(ψ)
    space_of(i, a) = if st.qb !== nothing
        (u1space(st.qb[i]) ⊗ MPSKit.physicalspace(ψ, i)) ← u1space(st.qb[i + 1])
    else
        (ComplexSpace(size(a, 1)) ⊗ MPSKit.physicalspace(ψ, i)) ← ComplexSpace(size(a, 3))
    end
    ac1 = st.AL[1] === nothing ?
          mul(context_of(st), :gb_mps_mul_front, st.C[1], st.AR[1],
              (st.C[1].dims[1], st.AR[1].dims[2], st.AR[1].dims[3]), T) :
          mul(context_of(st), :gb_mps_mul_tail, st.AL[1], st.C[2],
              (st.AL[1].dims[1], st.AL[1].dims[2], st.C[2].dims[2]), T)
    As = Vector{Any}(undef, n)
    a = download(ac1, T)
    As[1] = fromdense(a, space_of(1, a))
    for i in 2:n
        a = download(st.AR[i], T)
        As[i] = fromdense(a, space_of(i, a))
    end
    return FiniteMPS(As; normalize = false)
end
context_of(st::DeviceMPS) = st.ctx

# a U1 graded space with the given (2q) charges, in the sorted multiplicities they come in
function u1space(q::Vector{Int32})
    counts = Dict{Int32, Int}()
    foreach(c -> counts[c] = get(counts, c, 0) + 1, q)
    return U1Space((c // 2 => m for (c, m) in sort!(collect(counts)))...)
end

end # module
