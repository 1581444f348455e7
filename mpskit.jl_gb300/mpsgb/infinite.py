"""VUMPS on a one-site unit cell, with InfiniteMPOHamiltonian environments, on the device.

  InfiniteMPS gauge fixing (uniform_leftorth!/rightorth!) -- src/states/ortho.jl:210-340
  regauge!(AC, C)                                          -- src/states/ortho.jl:178-184
  InfiniteEnvironments for an InfiniteMPOHamiltonian      -- src/environments/infinite_envs.jl:177-346
  VUMPS                                                    -- src/algorithms/groundstate/vumps.jl:62-192

The environments are solved level by level (channel block by channel block of the MPO,
which is upper triangular): the inhomogeneous term is a sum of transfers of the lower
levels, and each level solves x - x T_ii = b by GMRES (regularised on identity levels).
Each level is one gb_env_linsolve call (restarted GMRES on the device).  The uniform gauge
iterations use the reference's acceleration (gauge_eigsolve_step!, ortho.jl:258-263,
322-324): from iteration 10 on, the boundary C is replaced by the dominant eigenvector of the
mixed transfer map before the QR/LQ step.
"""
import ctypes
import time

import numpy as np

from . import _lib as L
from .core import DeviceTensor, context
from .derivatives import GB300Backend, Lanczos, fixedpoint, integrate, DerivativeOperator
from .states import left_orth, mul_front, mul_tail, project_complement_, right_orth


def _dyn_tol(eps, it, factor, tmin=1e-14, tmax=1e-4):
    """DynamicTol with the Defaults bounds (src/utility/dynamictols.jl:86-89)."""
    return min(max(factor * eps / np.sqrt(max(it, 1)), tmin), tmax)


def _as_mps(C):
    """A bond tensor C[l; r] viewed as an MPS tensor with a trivial physical leg."""
    t = DeviceTensor(C.ctx, L.GB_KIND_MPS, C.dtype, (C.dims[0], 1, C.dims[1]))
    L.check(L.lib().gb_tensor_copy(t.handle, C.handle))
    return t


def _as_bond(A):
    t = DeviceTensor(A.ctx, L.GB_KIND_BOND, A.dtype, (A.dims[0], A.dims[2]))
    L.check(L.lib().gb_tensor_copy(t.handle, A.handle))
    return t


def adjoint(C):
    out = DeviceTensor(C.ctx, L.GB_KIND_BOND, C.dtype, (C.dims[1], C.dims[0]))
    L.check(L.lib().gb_tensor_adjoint(C.ctx.handle, C.handle, out.handle))
    return out


def _bond_mul(A, B):
    """A B for bond tensors."""
    return _as_bond(mul_tail(_as_mps(A), B))


def _diff_norm(a, b):
    t = a.copy()
    t.axpy_(-1.0, b)
    return t.norm()


class InfiniteMPS:
    """One-site unit cell on the device: AL C = C AR = AC."""

    def __init__(self, AL, AR, C):
        self.AL, self.AR, self.C = AL, AR, C

    @property
    def ctx(self):
        return self.C.ctx

    @property
    def dtype(self):
        return self.C.dtype

    @property
    def AC(self):
        return mul_tail(self.AL, self.C)

    @classmethod
    def from_tensor(cls, A, ctx=None, tol=1e-13, maxiter=200):
        """InfiniteMPS(A): left then right uniform gauge fixing (order :LR); A is a host
        array or a device MPS tensor."""
        if isinstance(A, DeviceTensor):
            ctx = A.ctx
        else:
            ctx = ctx or context()
            A = DeviceTensor.from_numpy(ctx, L.GB_KIND_MPS, A)
        D = A.dims[0]
        C0 = DeviceTensor.from_numpy(ctx, L.GB_KIND_BOND, np.eye(D, dtype=A.dtype))
        AL, C = uniform_leftorth(A, C0, tol, maxiter)
        AR, C = uniform_rightorth(AL, C, tol, maxiter)
        return cls(AL, AR, C)

    def to_numpy(self):
        return self.AL.numpy(), self.AR.numpy(), self.C.numpy()


def _transfer_bond(side, A, B, X):
    """side 0: sum_s B[s]' X A[s]; side 1: sum_s A[s] X B[s]' (gb_mps_transfer_bond)."""
    shape = (B.dims[2], A.dims[2]) if side == 0 else (A.dims[0], B.dims[0])
    out = DeviceTensor(X.ctx, L.GB_KIND_BOND, X.dtype, shape)
    L.check(L.lib().gb_mps_transfer_bond(X.ctx.handle, side, A.handle, B.handle, X.handle,
                                         out.handle))
    return out


def _arnoldi_dominant(op, x0, tol, krylovdim=30, maxiter=200):
    """Eigenvector of the largest-magnitude eigenvalue of `op` (KrylovKit Arnoldi, :LM, eager;
    explicit restarts from the Ritz vector).  The basis lives in one device tensor and every
    new vector is orthogonalised against it by two batched Gram-Schmidt passes
    (gb_basis_orthogonalize); the Hessenberg matrix and its eigenproblem stay on the host."""
    real = x0.dtype.kind != "c"
    ctx = x0.ctx
    n = int(np.prod(x0.dims))
    basis = DeviceTensor(ctx, L.GB_KIND_GENERIC, x0.dtype, (n, krylovdim + 1))
    h = np.zeros(2 * (krylovdim + 1))
    hp = h.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    x = x0.copy().normalize_()
    for _ in range(maxiter):
        L.check(L.lib().gb_basis_set(ctx.handle, basis.handle, 0, x.handle))
        Hm = np.zeros((krylovdim + 1, krylovdim), dtype=np.complex128)
        y = np.ones(1)
        v = x
        for j in range(krylovdim):
            w = op(v)
            L.check(L.lib().gb_basis_orthogonalize(ctx.handle, basis.handle, j + 1, w.handle, hp))
            Hm[:j + 1, j] = h[0:2 * (j + 1):2] + 1j * h[1:2 * (j + 1):2]
            hn = w.norm()
            Hm[j + 1, j] = hn
            k = j + 1
            ev, U = np.linalg.eig(Hm[:k, :k])
            i = int(np.argmax(np.abs(ev)))
            y = U[:, i] / np.linalg.norm(U[:, i])
            # an invariant subspace (hn at rounding level of H) ends the expansion
            breakdown = hn <= 1e-14 * max(1.0, np.linalg.norm(Hm[:k, :k]))
            if abs(hn * y[-1]) <= tol or breakdown:
                break
            v = w.scale_(1.0 / hn)
            L.check(L.lib().gb_basis_set(ctx.handle, basis.handle, k, v.handle))
        if real:
            y = y.real * np.sign(y.real[np.argmax(np.abs(y.real))])
        c = np.zeros(2 * len(y))
        c[0::2] = np.real(y)
        c[1::2] = 0.0 if real else np.imag(y)
        x = x0.similar()
        L.check(L.lib().gb_basis_combine(ctx.handle, basis.handle, len(y),
                                         c.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                         x.handle))
        x.normalize_()
        if abs(hn * y[-1]) <= tol or breakdown:
            break
    return x


def uniform_leftorth(A, C0, tol=1e-13, maxiter=200, eig_miniter=10):
    """uniform_leftorth! (src/states/ortho.jl:215-277): positive-QR iterations C A = AL C';
    from iteration eig_miniter on, C is first replaced by the dominant eigenvector of
    X -> sum_s AL[s]' X A[s] (Arnoldi, tolerance clamp(err^2, 1e-14, 1e-4)), made upper
    triangular by a positive QR -- the acceleration of gauge_eigsolve_step!."""
    C = C0.copy().normalize_()
    AL = None
    err = np.inf
    for it in range(maxiter):
        if it >= eig_miniter and AL is not None:
            t = min(max(err * err, 1e-14), 1e-4)
            vec = _arnoldi_dominant(lambda X: _transfer_bond(0, A, AL, X), C, t)
            _, C = left_orth(_as_mps(vec))
            C.normalize_()
        AL, R = left_orth(mul_front(C, A))
        R.normalize_()
        err = _diff_norm(C, R)
        C = R
        if err < tol:
            break
    return AL, C


def uniform_rightorth(A, C0, tol=1e-13, maxiter=200, eig_miniter=10):
    """uniform_rightorth! (src/states/ortho.jl:279-340): positive-LQ iterations A C = C' AR,
    accelerated from iteration eig_miniter on by the dominant eigenvector of
    X -> sum_s A[s] X AR[s]' (made lower triangular by a positive LQ)."""
    C = C0.copy().normalize_()
    AR = None
    err = np.inf
    for it in range(maxiter):
        if it >= eig_miniter and AR is not None:
            t = min(max(err * err, 1e-14), 1e-4)
            vec = _arnoldi_dominant(lambda X: _transfer_bond(1, A, AR, X), C, t)
            C, _ = right_orth(_as_mps(vec))
            C.normalize_()
        Lm, AR = right_orth(mul_tail(A, C))
        Lm.normalize_()
        err = _diff_norm(C, Lm)
        C = Lm
        if err < tol:
            break
    return AR, C


def regauge(AC, C):
    """AL = Q_AC Q_C' from positive QRs of AC and C."""
    qac, _ = left_orth(AC)
    qc, _ = left_orth(_as_mps(C))
    return mul_tail(qac, adjoint(_as_bond(qc)))


# ---------------------------------------------------------------- environments

def _levels(chans):
    off = np.concatenate([[0], np.cumsum(chans)]).astype(int)
    return [(int(off[i]), int(chans[i])) for i in range(len(chans))]


def _is_identity_block(B):
    n, d = B.shape[0], B.shape[1]
    ref = np.einsum("ab,st->astb", np.eye(n), np.eye(d))
    return B.shape == ref.shape and np.array_equal(B, ref)


class _Blocks:
    """Device copies of the nonzero MPO channel blocks W[level_j, :, :, level_i]."""

    def __init__(self, ctx, W, chans, dtype):
        self.lv = _levels(chans)
        self.W = W
        self.blk = {}
        for j, (oj, nj) in enumerate(self.lv):
            for i, (oi, ni) in enumerate(self.lv):
                b = W[oj:oj + nj, :, :, oi:oi + ni]
                if np.any(b != 0):
                    self.blk[(j, i)] = DeviceTensor.from_numpy(ctx, L.GB_KIND_MPO,
                                                               np.ascontiguousarray(b), dtype)

    def diag_kind(self, i):
        oi, ni = self.lv[i]
        d = self.W[oi:oi + ni, :, :, oi:oi + ni]
        if i == 0 or i == len(self.lv) - 1 or _is_identity_block(d):
            return "identity"
        return "diag" if (i, i) in self.blk else "empty"


def _transfer(side, ctx, env, Wb, A, prec):
    D = A.dims[2] if side == "L" else A.dims[0]
    out_w = Wb.dims[3] if side == "L" else Wb.dims[0]
    kind = L.GB_KIND_GL if side == "L" else L.GB_KIND_GR
    out = DeviceTensor(ctx, kind, env.dtype, (D, out_w, D))
    f = L.lib().gb_env_transfer_left if side == "L" else L.lib().gb_env_transfer_right
    L.check(f(ctx.handle, env.handle, Wb.handle, A.handle, A.handle, prec, out.handle))
    return out


def _regularize(ctx, x, lvec, rvec):
    """x -= tr(lvec x) rvec on every channel of the level block."""
    for c in range(x.dims[1]):
        L.check(L.lib().gb_env_regularize(ctx.handle, x.handle, c, lvec.handle, rvec.handle))
    return x


def _linsolve(side, ctx, b, x0, Wd, A, prec, reg, kd, maxiter, tol):
    """x - T(x) = b for one environment level on the device (gb_env_linsolve: KrylovKit
    linsolve(T, b, x0, GMRES, 1, -1), infinite_envs.jl:236-322); `reg` = (lvec, rvec) adds
    the regularisation of the identity levels.  Returns (x, converged, normres)."""
    x = x0.copy()
    ki = L.KrylovInfo()
    lv, rv = reg if reg is not None else (None, None)
    L.check(L.lib().gb_env_linsolve(ctx.handle, 0 if side == "L" else 1, Wd.handle, A.handle,
                                    prec, lv.handle if lv is not None else None,
                                    rv.handle if rv is not None else None, b.handle, x.handle,
                                    int(kd), int(maxiter), float(tol), ctypes.byref(ki)))
    return x, bool(ki.converged), ki.normres


class InfiniteEnvironments:
    """Fixed-point GL/GR of a one-site-cell InfiniteMPOHamiltonian on the device."""

    def __init__(self, psi, H, precision=L.GB_PREC_FP64):
        self.ctx = psi.ctx
        self.H = H
        self.dtype = np.result_type(psi.dtype, H.dtype)
        self.precision = precision
        self.blocks = _Blocks(self.ctx, H.W[0], H.chans[0], self.dtype)
        self.GLl = None  # per-level blocks (previous solutions are GMRES starting points)
        self.GRl = None
        self.GL = self.GR = None

    def recalculate(self, psi, tol=1e-12, krylovdim=30, maxiter=200):
        ctx, B, prec = self.ctx, self.blocks, self.precision
        lv = B.lv
        n = len(lv)
        D = psi.AL.dims[0]
        kd = min(D * D, krylovdim)
        eye = DeviceTensor.from_numpy(ctx, L.GB_KIND_BOND, np.eye(D, dtype=self.dtype))
        zero = lambda ni, kind: DeviceTensor.from_numpy(ctx, kind, np.zeros((D, ni, D), self.dtype))
        one = lambda kind: DeviceTensor.from_numpy(ctx, kind, np.eye(D, dtype=self.dtype)[:, None, :])
        r_LL = _bond_mul(psi.C, adjoint(psi.C))
        l_RR = _bond_mul(adjoint(psi.C), psi.C)
        prevL = self.GLl or [None] * n
        prevR = self.GRl or [None] * n
        # left levels, ascending
        GL = [one(L.GB_KIND_GL)] + [None] * (n - 1)
        for i in range(1, n):
            b = zero(lv[i][1], L.GB_KIND_GL)
            for j in range(i):
                if (j, i) in B.blk:
                    b.axpy_(1.0, _transfer("L", ctx, GL[j], B.blk[(j, i)], psi.AL, prec))
            x0 = prevL[i] if prevL[i] is not None else zero(lv[i][1], L.GB_KIND_GL)
            kind = B.diag_kind(i)
            if kind == "identity":
                Wd = B.blk[(i, i)]
                x, conv, nr = _linsolve("L", ctx, b, x0, Wd, psi.AL, prec, (r_LL, eye), kd,
                                        maxiter, tol)
                _regularize(ctx, x, r_LL, eye)
            elif kind == "diag":
                Wd = B.blk[(i, i)]
                x, conv, nr = _linsolve("L", ctx, b, x0, Wd, psi.AL, prec, None, kd, maxiter, tol)
            else:
                x = b
            GL[i] = x
        # right levels, descending
        GR = [None] * (n - 1) + [one(L.GB_KIND_GR)]
        for i in range(n - 2, -1, -1):
            b = zero(lv[i][1], L.GB_KIND_GR)
            for j in range(i + 1, n):
                if (i, j) in B.blk:
                    b.axpy_(1.0, _transfer("R", ctx, GR[j], B.blk[(i, j)], psi.AR, prec))
            x0 = prevR[i] if prevR[i] is not None else zero(lv[i][1], L.GB_KIND_GR)
            kind = B.diag_kind(i)
            if kind == "identity":
                Wd = B.blk[(i, i)]
                x, conv, nr = _linsolve("R", ctx, b, x0, Wd, psi.AR, prec, (l_RR, eye), kd,
                                        maxiter, tol)
                _regularize(ctx, x, l_RR, eye)
            elif kind == "diag":
                Wd = B.blk[(i, i)]
                x, conv, nr = _linsolve("R", ctx, b, x0, Wd, psi.AR, prec, None, kd, maxiter, tol)
            else:
                x = b
            GR[i] = x
        self.GLl, self.GRl = GL, GR
        w = sum(ni for _, ni in lv)
        self.GL = DeviceTensor(ctx, L.GB_KIND_GL, self.dtype, (D, w, D))
        self.GR = DeviceTensor(ctx, L.GB_KIND_GR, self.dtype, (D, w, D))
        for i, (oi, ni) in enumerate(lv):
            L.check(L.lib().gb_env_channel_copy(ctx.handle, self.GL.handle, oi, GL[i].handle, 0, ni))
            L.check(L.lib().gb_env_channel_copy(ctx.handle, self.GR.handle, oi, GR[i].handle, 0, ni))
        return self


def _heff_ac(envs, backend):
    W = envs.H.device(envs.ctx, envs.dtype)[0]
    return DerivativeOperator(envs.ctx, L.GB_HEFF_AC, envs.GL, W, None, envs.GR, backend)


def _heff_c(envs, backend):
    return DerivativeOperator(envs.ctx, L.GB_HEFF_C, envs.GL, None, None, envs.GR, backend)


def energy_density(psi, envs, backend=None):
    """expectation_value(::InfiniteMPS, ::InfiniteMPOHamiltonian) (expval.jl:150-161):
    <AC| GL . W[:, :, :, end] . GR[end] |AC>."""
    ctx = envs.ctx
    W = envs.H.W[0]
    wl = W.shape[0]
    Wl = DeviceTensor.from_numpy(ctx, L.GB_KIND_MPO, np.ascontiguousarray(W[:, :, :, -1:]),
                                 envs.dtype)
    D = envs.GR.dims[0]
    GRl = DeviceTensor(ctx, L.GB_KIND_GR, envs.dtype, (D, 1, D))
    L.check(L.lib().gb_env_channel_copy(ctx.handle, GRl.handle, 0, envs.GR.handle,
                                        envs.GR.dims[1] - 1, 1))
    op = DerivativeOperator(ctx, L.GB_HEFF_AC, envs.GL, Wl, None, GRl, backend or GB300Backend())
    ac = psi.AC
    return float(np.real(ac.dot(op(ac))))


def galerkin(psi, envs, backend=None):
    """calc_galerkin (toolbox.jl:63-70): |(1 - AL AL') normalize(H_AC(AC))|."""
    y = _heff_ac(envs, backend or GB300Backend())(psi.AC)
    y.normalize_()
    project_complement_(y, psi.AL)
    return y.norm()


class VUMPS:
    """VUMPS defaults (vumps.jl:19-43): tol 1e-10, maxiter 200, DynamicTol-adapted
    eigensolver (factor 1e-3), environment (1e-4) and gauge (1e-6) tolerances."""

    def __init__(self, tol=1e-10, maxiter=200, backend=None, verbosity=0):
        self.tol, self.maxiter = tol, maxiter
        self.backend = backend or GB300Backend()
        self.verbosity = verbosity


def find_groundstate_vumps(psi, H, alg, envs=None):
    """find_groundstate(::InfiniteMPS, H, VUMPS()) for a one-site cell (an InfiniteMPSCell
    goes to the cell form, `cell.find_groundstate_vumps`).  Returns (psi, envs, eps,
    history)."""
    from . import cell
    if isinstance(psi, cell.InfiniteMPSCell):
        return cell.find_groundstate_vumps(psi, H, alg, envs)
    envs = envs or InfiniteEnvironments(psi, H, alg.backend.code)
    it = 0
    envs.recalculate(psi, tol=1e-10)
    eps = galerkin(psi, envs, alg.backend)
    envs.recalculate(psi, tol=_dyn_tol(eps, it, 1e-4))
    hist = []
    clock = time.perf_counter
    while True:
        # phase wall times (every phase ends on a host read of a device result)
        t0 = clock()
        et = _dyn_tol(eps, it, 1e-3)
        solver = Lanczos(krylovdim=30, maxiter=200, tol=et, eager=True)
        _, AC, iac = fixedpoint(_heff_ac(envs, alg.backend), psi.AC, "SR", solver)
        t1 = clock()
        _, C, ic = fixedpoint(_heff_c(envs, alg.backend), psi.C, "SR", solver)
        t2 = clock()
        AL = regauge(AC, C)
        AR, C = uniform_rightorth(AL, psi.C, tol=_dyn_tol(eps, it, 1e-6))
        psi = InfiniteMPS(AL, AR, C)
        t3 = clock()
        envs.recalculate(psi, tol=_dyn_tol(eps, it, 1e-4))
        t4 = clock()
        eps = galerkin(psi, envs, alg.backend)
        it += 1
        e = energy_density(psi, envs, alg.backend)
        t5 = clock()
        hist.append({"iter": it, "energy": e, "eps": eps,
                     "phase_s": {"ac_eigsolve": t1 - t0, "c_eigsolve": t2 - t1,
                                 "gauge": t3 - t2, "environments": t4 - t3,
                                 "galerkin_energy": t5 - t4},
                     "matvecs": {"ac": iac.numops, "c": ic.numops}})
        if alg.verbosity:
            print(f"VUMPS {it}: e = {e:.14f}  eps = {eps:.3e}")
        if eps <= alg.tol or it >= alg.maxiter:
            break
    return psi, envs, eps, hist


class IDMRG:
    """IDMRG defaults (idmrg.jl:14-31): tol 1e-10, maxiter 200, DynamicTol-adapted
    eigensolver (factor 1e-3) and gauge (factor 1e-6) tolerances."""

    def __init__(self, tol=1e-10, maxiter=200, backend=None, verbosity=0):
        self.tol, self.maxiter = tol, maxiter
        self.backend = backend or GB300Backend()
        self.verbosity = verbosity


def find_groundstate_idmrg(psi, H, alg, envs=None):
    """find_groundstate(::InfiniteMPS, H, IDMRG()) for a one-site cell (idmrg.jl:85-216).
    Per iteration: AC eigensolve, positive QR AC = AL C, GL <- GL T(AL) (un-normalised,
    transfer_leftenv!, infinite_envs.jl:359-363); AC eigensolve again, positive LQ
    AC = C AR, GR <- T(AR) GR; error |C - C_old|.  The result is InfiniteMPS(AR) with the
    DynamicTol gauge tolerance and recalculated environments.  Returns (psi, envs, eps,
    history); history entries carry the energy change per site (E - E_old) / 2.  An
    InfiniteMPSCell goes to the cell form (`cell.find_groundstate_idmrg`)."""
    from . import cell
    if isinstance(psi, cell.InfiniteMPSCell):
        return cell.find_groundstate_idmrg(psi, H, alg, envs)
    envs = envs or InfiniteEnvironments(psi, H, alg.backend.code)
    ctx = psi.ctx
    envs.recalculate(psi, tol=1e-10)  # environments(psi, H): GMRES at Defaults.tol
    eps = galerkin(psi, envs, alg.backend)
    E_old = energy_density(psi, envs, alg.backend)
    W = H.device(ctx, envs.dtype)[0]
    AC, C, AR = psi.AC, psi.C, psi.AR
    it = 0
    hist = []
    while True:
        solver = Lanczos(krylovdim=30, maxiter=200, tol=_dyn_tol(eps, it, 1e-3), eager=True)
        C_old = C
        _, AC, _ = fixedpoint(_heff_ac(envs, alg.backend), AC, "SR", solver)
        AL, _ = left_orth(AC)
        envs.GL = _transfer("L", ctx, envs.GL, W, AL, envs.precision)
        E, AC, _ = fixedpoint(_heff_ac(envs, alg.backend), AC, "SR", solver)
        C, AR = right_orth(AC)
        envs.GR = _transfer("R", ctx, envs.GR, W, AR, envs.precision)
        eps = _diff_norm(C, C_old)
        it += 1
        hist.append({"iter": it, "energy_change": (E - E_old) / 2, "eps": eps})
        E_old = E
        if alg.verbosity:
            print(f"IDMRG {it}: dE = {hist[-1]['energy_change']:.14f}  eps = {eps:.3e}")
        if eps <= alg.tol or it >= alg.maxiter:
            break
    psi = InfiniteMPS.from_tensor(AR, tol=_dyn_tol(eps, it, 1e-6), maxiter=200)
    envs.recalculate(psi, tol=1e-10)
    return psi, envs, eps, hist


def timestep_infinite(psi, H, t, dt, alg=None, envs=None, imaginary_evolution=False,
                      tolgauge=1e-14):
    """timestep(::InfiniteMPS, H, t, dt, TDVP()) for a one-site cell (tdvp.jl:72-133,
    leftorthflag = true): AC and C are integrated with the same environments, AL =
    regauge(AC, C), the state is rebuilt by the uniform right gauge from AL (old C as the
    starting point) and the environments are recalculated.  Returns (psi, envs).  An
    InfiniteMPSCell goes to the cell form (`cell.timestep`)."""
    from . import cell
    if isinstance(psi, cell.InfiniteMPSCell):
        return cell.timestep(psi, H, t, dt, alg, envs, imaginary_evolution, tolgauge)
    from .algorithms import TDVP
    alg = alg or TDVP()
    if psi.dtype.kind != "c" and not imaginary_evolution:
        raise TypeError("real-time evolution needs a complex InfiniteMPS")
    if envs is None:
        envs = InfiniteEnvironments(psi, H, alg.backend.code)
    if envs.GL is None:
        envs.recalculate(psi)
    AC = integrate(_heff_ac(envs, alg.backend), psi.AC, t, dt, alg.integrator,
                   imaginary_evolution)
    C = integrate(_heff_c(envs, alg.backend), psi.C, t, dt, alg.integrator, imaginary_evolution)
    AL = regauge(AC, C)
    AR, C = uniform_rightorth(AL, psi.C, tol=tolgauge)
    psi = InfiniteMPS(AL, AR, C)
    envs.recalculate(psi)
    return psi, envs
