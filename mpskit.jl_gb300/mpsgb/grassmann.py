"""GradientGrassmann on the device (finite MPS, one-site InfiniteMPS and InfiniteMPS unit
cells): the left-canonical tensors AL[i] as points of Grassmann manifolds, optimised by
Riemannian conjugate gradients (mpsgb.optim).

  GradientGrassmann, find_groundstate  -- src/algorithms/groundstate/gradient_grassmann.jl:1-121
  fg, precondition, retract, transport, inner, rho_inv_regularized
                                       -- src/algorithms/grassmann.jl:1-262

The tangent-space geometry is that of TensorKitManifolds.Grassmann (compat 0.7, 0.8, outside
the reference sources); it is restated from the geodesic and parallel-transport formulas of
A. Edelman, T. A. Arias, S. T. Smith, "The geometry of algorithms with orthogonality
constraints", SIAM J. Matrix Anal. Appl. 20 (1998) 303-353, eqs. (2.65) and (2.68): for a
point W and a tangent Z = U S V' (compact SVD),

  W(a)        = W + (W V (cos aS - 1) + U sin aS) V'
  Z(a)        = (-W V sin aS + U cos aS) S V'            (the direction carried along)
  T_a(Theta)  = Theta + (-W V sin aS + U (cos aS - 1)) U' Theta

with W(a) replaced by its polar factor (projectisometric) and each new tangent projected
onto the complement of the new point (removing rounding).

Every tensor operation runs in libmpsgb (gemm-backed MPS products, the positive QR/LQ
gauge, the cuSOLVER SVD of the tangent and bond matrices, the Jordan AC derivative); the
host keeps only scalars and the singular values that scale the bond directions.
"""
import ctypes
from dataclasses import dataclass, field

import numpy as np

from . import _lib as L
from .core import DeviceTensor
from .derivatives import AC_hamiltonian, GB300Backend
from .infinite import adjoint
from .optim import ConjugateGradient, HagerZhangLineSearch, optimize
from .states import (FiniteEnvironments, FiniteMPS, left_orth, mul_front, mul_tail,
                     project_complement_, svd_trunc)


# ------------------------------------------------------------------ small device helpers
def _diag(ctx, v, dtype):
    return DeviceTensor.from_numpy(ctx, L.GB_KIND_BOND, np.diag(np.asarray(v, dtype=dtype)))


def _svd(M, dims):
    """Compact SVD of a device matrix viewed as the (first legs) x (last leg) matrix of an
    MPS tensor `dims` = (Dl, d, Dr): U (Dl, d, k) as an MPS tensor, host singular values s
    (k), Vh (k, Dr) as a bond tensor.  cuSOLVER gesvd through gb_svd_trunc with no
    truncation."""
    ctx = M.ctx
    Dl, d, Dr = dims
    a = M.copy().reshape_(L.GB_KIND_AC2, (Dl, d, Dr, 1))
    saved = getattr(ctx, "_svd_method", "gesvd")
    ctx.set_svd_method("gesvd")
    try:
        U, S, Vh, _ = svd_trunc(a, None, 0.0, normalize=False)
    finally:
        if saved != "gesvd":
            ctx.set_svd_method(saved)
    s = np.real(np.diag(S.numpy())).copy()
    Vb = Vh.copy().reshape_(L.GB_KIND_BOND, (Vh.dims[0], Vh.dims[2]))
    return U, s, Vb


def _svd_batch(ts):
    """Compact SVDs of several tall device matrices in one call (gb_svd_batch, on the
    context's lanes): [(U, s, Vh)] with U of each input's kind, s on the host, Vh a bond."""
    if not ts:
        return []
    ctx = ts[0].ctx
    n = len(ts)
    hv = lambda h: h.value if isinstance(h, ctypes.c_void_p) else h
    arr = (ctypes.c_void_p * n)(*[hv(t.handle) for t in ts])
    U, V = (ctypes.c_void_p * n)(), (ctypes.c_void_p * n)()
    S = np.zeros(sum(t.dims[-1] for t in ts))
    L.check(L.lib().gb_svd_batch(ctx.handle, n, arr, U, V,
                                 S.ctypes.data_as(ctypes.POINTER(ctypes.c_double))))
    out, off = [], 0
    for i, t in enumerate(ts):
        k = t.dims[-1]
        out.append((DeviceTensor.wrap(ctx, ctypes.c_void_p(U[i])), S[off:off + k].copy(),
                    DeviceTensor.wrap(ctx, ctypes.c_void_p(V[i]))))
        off += k
    return out


def _fill_svds(tangents):
    """Factorise every tangent whose SVD is not cached yet, all in one batch."""
    todo = [t for t in tangents if t._svd is None]
    for t, r in zip(todo, _svd_batch([t.Z for t in todo])):
        t._svd = r


def _bond_as_mps(C):
    return C.copy().reshape_(L.GB_KIND_MPS, (C.dims[0], 1, C.dims[1]))


def _mps_as_bond(A):
    return A.copy().reshape_(L.GB_KIND_BOND, (A.dims[0] * A.dims[1], A.dims[2]))


def _left_overlap(U, Z):
    """U' Z over the first two legs: (k x Dr) = sum_(l s) conj(U[l s; k]) Z[l s; r]."""
    ctx = U.ctx
    Dl, d, k = U.dims
    one = DeviceTensor.from_numpy(ctx, L.GB_KIND_BOND, np.ones((1, 1), dtype=U.dtype))
    Uf = U.copy().reshape_(L.GB_KIND_MPS, (1, Dl * d, k))
    Zf = Z.copy().reshape_(L.GB_KIND_MPS, (1, Dl * d, Z.dims[2]))
    out = DeviceTensor(ctx, L.GB_KIND_BOND, Z.dtype, (k, Z.dims[2]))
    L.check(L.lib().gb_mps_transfer_bond(ctx.handle, 0, Zf.handle, Uf.handle, one.handle,
                                         out.handle))
    return out


# ------------------------------------------------------------------ tangent vectors
class GrassmannTangent:
    """Tangent Z at the point W (Z' W = 0), with its compact SVD cached."""

    __slots__ = ("W", "Z", "_svd")

    def __init__(self, W, Z):
        self.W, self.Z, self._svd = W, Z, None

    def svd(self):
        if self._svd is None:
            self._svd = _svd_batch([self.Z])[0]
        return self._svd

    def norm(self):
        return self.Z.norm()


def project(X, W):
    """Grassmann.project: the tangent part X - W (W' X) of X at W."""
    return GrassmannTangent(W, project_complement_(X.copy(), W))


def polar_factor(W, maxiter=6):
    """The unitary polar factor of a near-isometry W (its columns), the projectisometric
    of the retraction, by Newton-Schulz iterations W <- W (3 - W'W) / 2 (quadratic
    convergence to the polar factor while |W'W - 1| < 1): GEMMs only, no SVD.  Stops once
    |W'W - 1| is at rounding level; falls back to the SVD (U V') if the iteration does not
    settle."""
    ctx, k = W.ctx, W.dims[2]
    eye = DeviceTensor.from_numpy(ctx, L.GB_KIND_BOND, np.eye(k, dtype=W.dtype))
    for _ in range(maxiter):
        G = _left_overlap(W, W)
        G.axpy_(-1.0, eye)
        err = float(np.abs(G.numpy()).max())
        if err <= 4.0 * np.finfo(np.float64).eps * k:
            return W
        if err >= 0.5:
            break
        G.scale_(-0.5)
        G.axpy_(1.0, eye)          # (3 - W'W) / 2 = 1 - (W'W - 1) / 2
        W = mul_tail(W, G)
    U, _, Vh = _svd(W, W.dims)
    return mul_tail(U, Vh)


def retract_site(W, D, a):
    """Grassmann.retract(W, D, a) -> (W(a), D(a)): the geodesic from W along D."""
    ctx, dt = W.ctx, W.dtype
    U, s, Vh = D.svd()
    WV = mul_tail(W, adjoint(Vh))
    cs, sn = np.cos(a * s), np.sin(a * s)
    T = mul_tail(WV, _diag(ctx, cs - 1.0, dt))
    T.axpy_(1.0, mul_tail(U, _diag(ctx, sn, dt)))
    Wn = W.copy()
    Wn.axpy_(1.0, mul_tail(T, Vh))
    # projectisometric: the polar factor.  Directions carry rounding noise off the tangent
    # space (most of all where the tangent space is empty and the preconditioner large);
    # without this the AL drift away from isometries over the iterations.
    Wn = polar_factor(Wn)
    T = mul_tail(WV, _diag(ctx, -sn * s, dt))
    T.axpy_(1.0, mul_tail(U, _diag(ctx, cs * s, dt)))
    Zn = project_complement_(mul_tail(T, Vh), Wn)
    return Wn, GrassmannTangent(Wn, Zn)


def transport_site(Th, W, D, a, Wn):
    """Grassmann.transport!(Th, W, D, a, Wn): parallel transport of Th along the geodesic
    of D (an isometry of the tangent spaces)."""
    ctx, dt = W.ctx, W.dtype
    U, s, Vh = D.svd()
    WV = mul_tail(W, adjoint(Vh))
    T = mul_tail(WV, _diag(ctx, -np.sin(a * s), dt))
    T.axpy_(1.0, mul_tail(U, _diag(ctx, np.cos(a * s) - 1.0, dt)))
    Z = Th.Z.copy()
    Z.axpy_(1.0, mul_tail(T, _left_overlap(U, Th.Z)))
    return GrassmannTangent(Wn, project_complement_(Z, Wn))


def rho_inv_regularized(C, rtol, svd=None):
    """U (S^2 + delta^2)^-1 U' with C = U S V' and delta = rtol * max(S) (Tikhonov
    regularised inverse of rho = C C', grassmann.jl:243-255); `svd` = (U, s, Vh) of C when
    already computed."""
    ctx, dt = C.ctx, C.dtype
    U, s, _ = svd if svd is not None else _svd_batch([C])[0]
    d2 = (rtol * (s.max() if s.size else 0.0)) ** 2
    Um = _bond_as_mps(U)
    return _mps_as_bond(mul_tail(mul_tail(Um, _diag(ctx, 1.0 / (s * s + d2), dt)),
                                 adjoint(U)))


# ------------------------------------------------------------------ points
class GrassmannPoint:
    """A finite MPS as its left-canonical tensors AL[0..L-1] and the 1 x 1 norm factor of
    the last bond; the bond matrices C (right of each site) and the right-canonical AR come
    from the positive LQ sweep, as the reference computes them lazily."""

    def __init__(self, AL, Cend):
        n = len(AL)
        C = [None] * (n + 1)
        C[n] = Cend
        self.psi = FiniteMPS(list(AL), [None] * n, C, n)
        self.psi.right_canonicalize(0)

    @classmethod
    def from_state(cls, psi):
        """The point of a FiniteMPS: its AL left of the centre bond, then positive QR moves
        through the right-canonical part; the remaining norm factor is normalised."""
        n, c = len(psi), psi.center
        AL = list(psi.AL[:c]) + [None] * (n - c)
        X = psi.C[c]
        for i in range(c, n):
            AL[i], X = left_orth(mul_front(X, psi.AR[i]))
        return cls(AL, X.copy().normalize_())

    def __len__(self):
        return len(self.psi.AL)

    @property
    def AL(self):
        return self.psi.AL

    def C_right(self, i):
        """MPSKit's C[i]: the bond matrix right of site i."""
        return self.psi.C[i + 1]


# ------------------------------------------------------------------ GrassmannMPS functions
def inner(x, g1, g2):
    """2 Re sum_i <Z1_i, Z2_i> (grassmann.jl:61-71)."""
    return 2.0 * sum(float(np.real(a.Z.dot(b.Z))) for a, b in zip(g1, g2))


def precondition(x, g):
    """g_i -> g_i rho_i^-1 with rho = C C' Tikhonov-regularised at
    max(eps^(3/4), |g_i|) (grassmann.jl:73-91)."""
    rtolmin = np.finfo(np.float64).eps ** 0.75
    svds = _svd_batch([x.C_right(i) for i in range(len(g))])
    out = []
    for i, gi in enumerate(g):
        rtol = max(rtolmin, gi.norm())
        rho = rho_inv_regularized(x.C_right(i), rtol, svds[i])
        out.append(GrassmannTangent(gi.W, mul_tail(gi.Z, rho)))
    return out


def retract(x, g, a):
    """retract(state::FiniteMPS, g, a) (grassmann.jl:93-108): every AL[i] along its
    geodesic; the new state keeps the old norm factor of the last bond, normalised."""
    _fill_svds(g)
    res = [retract_site(x.AL[i], g[i], a) for i in range(len(x))]
    Cend = x.psi.C[len(x)].copy().normalize_()
    return GrassmannPoint([r[0] for r in res], Cend), [r[1] for r in res]


def transport(h, x, g, a, xn):
    """transport!(h, state, g, a, state') (grassmann.jl:124-136)."""
    _fill_svds(g)
    return [transport_site(h[i], x.AL[i], g[i], a, xn.AL[i]) for i in range(len(x))]


def add(v, w, a, b):
    out = []
    for vi, wi in zip(v, w):
        z = vi.Z.copy().scale_(a)
        z.axpy_(b, wi.Z)
        out.append(GrassmannTangent(vi.W, z))
    return out


def scale(v, a):
    return [GrassmannTangent(vi.W, vi.Z.copy().scale_(a)) for vi in v]


def fg(x, H, envs, backend=None):
    """fg(state::FiniteMPS, H, envs) (grassmann.jl:150-169): the energy and, per site, the
    projected AC derivative Grassmann.project(AC_projection(i), AL[i]) times C[i]'."""
    backend = backend or GB300Backend()
    psi = x.psi
    AC0 = psi.ac(0)
    H0 = AC_hamiltonian(0, psi, H, envs, backend)
    f = AC0.dot(H0(AC0))
    f = complex(f) / AC0.norm() ** 2
    gs = []
    for i in range(len(x)):
        Ci = x.C_right(i)
        AC = mul_tail(psi.AL[i], Ci)
        y = AC_hamiltonian(i, psi, H, envs, backend)(AC)
        gi = project(y, psi.AL[i])
        gs.append(GrassmannTangent(gi.W, mul_tail(gi.Z, adjoint(Ci))))
    return float(np.real(f)), gs


# ------------------------------------------------------------------ driver
@dataclass
class GradientGrassmann:
    """GradientGrassmann(; method = ConjugateGradient, tol, maxiter, verbosity)
    (gradient_grassmann.jl:31-78): a ConjugateGradient with the Hager-Zhang line search
    capped at 100 evaluations, stopping at |g| <= tol or `maxiter` iterations."""
    tol: float = 1e-10         # Defaults.tol (src/utility/defaults.jl:25)
    maxiter: int = 200         # Defaults.maxiter (defaults.jl:23)
    verbosity: int = 0
    backend: GB300Backend = field(default_factory=GB300Backend)
    method: ConjugateGradient = None

    def __post_init__(self):
        if self.method is None:
            self.method = ConjugateGradient(gradtol=self.tol, maxiter=self.maxiter,
                                            linesearch=HagerZhangLineSearch(maxiter=100),
                                            verbosity=self.verbosity)


# ------------------------------------------------------------------ one-site InfiniteMPS
def fg_infinite(x, H, envs, backend=None):
    """fg(state::InfiniteMPS, H::InfiniteMPOHamiltonian, envs) (grassmann.jl:171-190): the
    fixed-point environments recalculated, the energy density, and the projected AC
    derivative times C'."""
    from .infinite import _heff_ac, energy_density
    backend = backend or GB300Backend()
    envs.recalculate(x)
    f = energy_density(x, envs, backend)
    y = _heff_ac(envs, backend)(x.AC)
    g = project(y, x.AL)
    return f, [GrassmannTangent(x.AL, mul_tail(g.Z, adjoint(x.C)))]


def retract_infinite(x, g, a):
    """retract(state::InfiniteMPS, g, a) (grassmann.jl:109-122): AL along its geodesic, then
    InfiniteMPS(AL', C) -- the right uniform gauge fixed from the old C."""
    from .infinite import InfiniteMPS, uniform_rightorth
    ALn, xi = retract_site(x.AL, g[0], a)
    AR, C = uniform_rightorth(ALn, x.C)
    return InfiniteMPS(ALn, AR, C), [xi]


def transport_infinite(h, x, g, a, xn):
    return [transport_site(h[0], x.AL, g[0], a, xn.AL)]


def precondition_infinite(x, g):
    rtol = max(np.finfo(np.float64).eps ** 0.75, g[0].norm())
    return [GrassmannTangent(g[0].W, mul_tail(g[0].Z, rho_inv_regularized(x.C, rtol)))]


# ------------------------------------------------------------------ InfiniteMPS, L-site cell
def fg_cell(x, H, envs, backend=None):
    """fg(state::InfiniteMPS, H::InfiniteMPOHamiltonian, envs) (grassmann.jl:171-190) for an
    L-site cell: the cell's fixed-point environments recalculated, the energy of the cell
    (expectation_value sums its sites, expval.jl:150-161) and per site the projected AC
    derivative times C[s]'."""
    from .cell import _heff_ac, energy
    backend = backend or GB300Backend()
    envs.recalculate(x)
    f = energy(x, envs)
    gs = []
    for s in range(len(x)):
        g = project(_heff_ac(envs, s, backend)(x.AC(s)), x.AL[s])
        gs.append(GrassmannTangent(x.AL[s], mul_tail(g.Z, adjoint(x.C[s]))))
    return f, gs


def retract_cell(x, g, a):
    """retract(state::InfiniteMPS, g, a) (grassmann.jl:106-115): every AL[s] along its
    geodesic, then InfiniteMPS(AL', C[end]) -- the cell's right uniform gauge."""
    from .cell import InfiniteMPSCell, uniform_rightorth
    out = [retract_site(x.AL[s], g[s], a) for s in range(len(x))]
    ALn = [o[0] for o in out]
    AR, C = uniform_rightorth(ALn, x.C[-1])
    return InfiniteMPSCell(ALn, AR, C), [o[1] for o in out]


def transport_cell(h, x, g, a, xn):
    return [transport_site(h[s], x.AL[s], g[s], a, xn.AL[s]) for s in range(len(x))]


def precondition_cell(x, g):
    """precondition(state, g) (grassmann.jl:85-94): g[s] rho_inv_regularized(C[s]) with the
    bond SVDs of the cell batched."""
    rtolmin = np.finfo(np.float64).eps ** 0.75
    svds = _svd_batch(list(x.C))
    return [GrassmannTangent(gs.W, mul_tail(gs.Z, rho_inv_regularized(
        x.C[s], max(rtolmin, gs.norm()), svds[s]))) for s, gs in enumerate(g)]


def find_groundstate_grassmann(psi, H, alg=None, envs=None):
    """find_groundstate(psi, H, GradientGrassmann) (gradient_grassmann.jl:80-121) ->
    (psi, envs, normgrad, history): the optimised state (finite: left-canonical, centre bond
    0 after the closing LQ sweep; infinite: uniformly gauged), its environments, the final
    gradient norm and the gradient-norm history."""
    alg = alg or GradientGrassmann()
    from .cell import InfiniteEnvironmentsCell, InfiniteMPSCell
    from .infinite import InfiniteEnvironments, InfiniteMPS
    if isinstance(psi, InfiniteMPSCell):
        envs = envs or InfiniteEnvironmentsCell(psi, H, alg.backend.code)
        x, f, g, numfg, hist = optimize(
            lambda x_: fg_cell(x_, H, envs, alg.backend), psi, alg.method, retract_cell,
            transport_cell, inner, add, scale, precondition_cell)
        envs.recalculate(x)
        return x, envs, hist[-1], {"energy": f / len(x), "energy_cell": f, "numfg": numfg,
                                   "normgrad": hist}
    if isinstance(psi, InfiniteMPS):
        envs = envs or InfiniteEnvironments(psi, H)
        x, f, g, numfg, hist = optimize(
            lambda x_: fg_infinite(x_, H, envs, alg.backend), psi, alg.method,
            retract_infinite, transport_infinite, inner, add, scale, precondition_infinite)
        envs.recalculate(x)
        return x, envs, hist[-1], {"energy": f, "numfg": numfg, "normgrad": hist}
    if psi.C[psi.center].charges is not None or (psi.AR[0] is not None
                                                 and psi.AR[0].charges is not None):
        raise NotImplementedError("GradientGrassmann: U(1)-charged states are not supported")
    x0 = GrassmannPoint.from_state(psi)
    if x0.psi.C[len(x0)].dims != (1, 1):
        raise ValueError("GradientGrassmann needs a state with a trivial last bond")
    envs = envs or FiniteEnvironments(x0.psi, H, psi.ctx)
    x, f, g, numfg, hist = optimize(
        lambda x_: fg(x_, H, envs, alg.backend), x0, alg.method, retract, transport, inner,
        add, scale, precondition)
    return x.psi, envs, hist[-1], {"energy": f, "numfg": numfg, "normgrad": hist}
