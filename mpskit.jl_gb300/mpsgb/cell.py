"""InfiniteMPS with a unit cell of L >= 1 sites on the device: uniform gauge, environments,
VUMPS, IDMRG, IDMRG2 and TDVP time steps.

  uniform_leftorth! / uniform_rightorth! over the cell  -- src/states/ortho.jl:214-340
  compute_leftenvs! / compute_rightenvs!, left_cyclethrough! / right_cyclethrough!
                                                         -- src/environments/infinite_envs.jl:207-346
  VUMPS (per-site AC and C eigensolves, gauge step, environments)
                                                         -- src/algorithms/groundstate/vumps.jl:101-192
  IDMRG (one-site sweeps through the cell)              -- src/algorithms/groundstate/idmrg.jl:85-229
  TDVP timestep (per-site AC and C integration)          -- src/algorithms/timestep/tdvp.jl:72-133
  IDMRG2 (two-site sweeps with the edge updates)        -- src/algorithms/groundstate/idmrg.jl:143-338

Sites are counted from 0; C[i] is the bond tensor right of site i and C[-1] = C[L-1] the one
at the cell boundary.  Everything runs through the same device operations as the one-site
path: environment transfers per MPO level block, the derivative operators and their Krylov
solvers, the positive QR/LQ and the truncated SVD.  A level of the environments is solved
at the cell boundary with the product transfer matrix of the whole cell; its GMRES runs on
the host over device vectors (one transfer per site per Krylov step).
"""
import numpy as np

from . import _lib as L
from .core import DeviceTensor, context
from .derivatives import (GB300Backend, Lanczos, DerivativeOperator, fixedpoint)
from .infinite import (_arnoldi_dominant, _as_mps, _diff_norm, _dyn_tol, _is_identity_block,
                       _levels, _regularize, _transfer, _transfer_bond, regauge)
from .states import ac2_from, left_orth, mul_front, mul_tail, project_complement_, right_orth
from .states import svd_trunc


class InfiniteMPSCell:
    """AL[i] C[i] = C[i-1] AR[i] = AC[i] for i in 0..L-1 (device tensors)."""

    def __init__(self, AL, AR, C):
        self.AL, self.AR, self.C = list(AL), list(AR), list(C)

    def __len__(self):
        return len(self.AL)

    @property
    def ctx(self):
        return self.C[0].ctx

    @property
    def dtype(self):
        return self.C[0].dtype

    def AC(self, i):
        return mul_tail(self.AL[i], self.C[i])

    @classmethod
    def from_tensors(cls, As, ctx=None, tol=1e-13, maxiter=200):
        """InfiniteMPS(As): left then right uniform gauge fixing (order :LR)."""
        if isinstance(As[0], DeviceTensor):
            ctx = As[0].ctx
        else:
            ctx = ctx or context()
            As = [DeviceTensor.from_numpy(ctx, L.GB_KIND_MPS, a) for a in As]
        D = As[0].dims[0]
        C0 = DeviceTensor.from_numpy(ctx, L.GB_KIND_BOND, np.eye(D, dtype=As[0].dtype))
        AL, C = uniform_leftorth(As, C0, tol, maxiter)
        AR, C = uniform_rightorth(AL, C[-1], tol, maxiter)
        return cls(AL, AR, C)

    def to_numpy(self):
        return ([a.numpy() for a in self.AL], [a.numpy() for a in self.AR],
                [c.numpy() for c in self.C])


def _cell_left_bond(As, Bs, X):
    """X -> sum over the cell of B' X A, site 0 first (flip(TransferMatrix(A, B)))."""
    for a, b in zip(As, Bs):
        X = _transfer_bond(0, a, b, X)
    return X


def _cell_right_bond(As, Bs, X):
    """X -> A X B' through the cell, the last site first (TransferMatrix(A, B))."""
    for a, b in zip(reversed(As), reversed(Bs)):
        X = _transfer_bond(1, a, b, X)
    return X


def uniform_leftorth(As, C0, tol=1e-13, maxiter=200, eig_miniter=10):
    """uniform_leftorth! over the cell: C[i-1] A[i] = AL[i] C[i] (positive QR) for i = 0..L-1,
    the boundary C normalised; from iteration eig_miniter on the boundary C is first replaced
    by the dominant eigenvector of the cell's mixed transfer map (gauge_eigsolve_step!)."""
    n = len(As)
    AL = [None] * n
    C = [None] * n
    C[n - 1] = C0.copy().normalize_()
    err = np.inf
    for it in range(maxiter):
        if it >= eig_miniter and AL[0] is not None:
            t = min(max(err * err, 1e-14), 1e-4)
            vec = _arnoldi_dominant(lambda X: _cell_left_bond(As, AL, X), C[n - 1], t)
            _, C[n - 1] = left_orth(_as_mps(vec))
            C[n - 1].normalize_()
        before = C[n - 1]
        for i in range(n):
            AL[i], C[i] = left_orth(mul_front(C[i - 1], As[i]))
        C[n - 1].normalize_()
        err = _diff_norm(before, C[n - 1])
        if err < tol:
            break
    return AL, C


def uniform_rightorth(As, C0, tol=1e-13, maxiter=200, eig_miniter=10):
    """uniform_rightorth! over the cell: A[i] C[i] = C[i-1] AR[i] (positive LQ) for
    i = L-1..0, accelerated like uniform_leftorth."""
    n = len(As)
    AR = [None] * n
    C = [None] * n
    C[n - 1] = C0.copy().normalize_()
    err = np.inf
    for it in range(maxiter):
        if it >= eig_miniter and AR[0] is not None:
            t = min(max(err * err, 1e-14), 1e-4)
            vec = _arnoldi_dominant(lambda X: _cell_right_bond(As, AR, X), C[n - 1], t)
            C[n - 1], _ = right_orth(_as_mps(vec))
            C[n - 1].normalize_()
        before = C[n - 1]
        for i in range(n - 1, -1, -1):
            C[i - 1], AR[i] = right_orth(mul_tail(As[i], C[i]))
        C[n - 1].normalize_()
        err = _diff_norm(before, C[n - 1])
        if err < tol:
            break
    return AR, C


def _gmres(op, b, x0, krylovdim=30, maxiter=200, tol=1e-12):
    """x - op(x) = b by restarted GMRES over device vectors (KrylovKit GMRES with a0 = 1,
    a1 = -1, as linsolve(T, b, x0, alg, 1, -1) is called by compute_leftenvs!)."""
    x = x0.copy()
    nb = b.norm()
    if nb == 0.0:
        x.scale_(0.0)
        return x, True

    def A(v):
        y = v.copy()
        y.axpy_(-1.0, op(v))
        return y

    for _ in range(maxiter):
        r = b.copy()
        r.axpy_(-1.0, A(x))
        beta = r.norm()
        if beta <= tol * max(1.0, nb):
            return x, True
        V = [r.scale_(1.0 / beta)]
        Hm = np.zeros((krylovdim + 1, krylovdim), dtype=np.complex128)
        k = 0
        for j in range(krylovdim):
            w = A(V[j])
            for _pass in range(2):
                for i in range(j + 1):
                    h = V[i].dot(w)
                    Hm[i, j] += h
                    w.axpy_(-h, V[i])
            hn = w.norm()
            Hm[j + 1, j] = hn
            k = j + 1
            e1 = np.zeros(k + 1, dtype=np.complex128)
            e1[0] = beta
            y, *_ = np.linalg.lstsq(Hm[:k + 1, :k], e1, rcond=None)
            res = np.linalg.norm(Hm[:k + 1, :k] @ y - e1)
            if res <= tol * max(1.0, nb) or hn <= 1e-14 * beta:
                break
            V.append(w.scale_(1.0 / hn))
        real = x.dtype.kind != "c"
        for i in range(k):
            x.axpy_(float(y[i].real) if real else complex(y[i]), V[i])
    r = b.copy()
    r.axpy_(-1.0, A(x))
    return x, r.norm() <= tol * max(1.0, nb)


class InfiniteEnvironmentsCell:
    """Fixed-point GL[s] / GR[s] of every site of the cell (the left and right environments
    of site s, on the bonds left and right of it)."""

    def __init__(self, psi, H, precision=L.GB_PREC_FP64):
        self.ctx = psi.ctx
        self.H = H
        self.n = len(psi)
        if len(H) != self.n:
            raise ValueError("the Hamiltonian's unit cell differs from the state's")
        self.dtype = np.result_type(psi.dtype, H.dtype)
        self.precision = precision
        self.lv = [_levels(H.chans[s]) for s in range(self.n + 1)]
        self.nlev = len(self.lv[0])
        # nonzero level blocks W[s][level j (left bond), :, :, level i (right bond)]
        self.blk = []
        for s in range(self.n):
            d = {}
            for j, (oj, nj) in enumerate(self.lv[s]):
                for i, (oi, ni) in enumerate(self.lv[s + 1]):
                    b = H.W[s][oj:oj + nj, :, :, oi:oi + ni]
                    if np.any(b != 0):
                        d[(j, i)] = (DeviceTensor.from_numpy(self.ctx, L.GB_KIND_MPO,
                                                             np.ascontiguousarray(b), self.dtype), b)
            self.blk.append(d)
        self.GLl = self.GRl = None
        self.GL = self.GR = None

    def _kind(self, i):
        """isidentitylevel / isemptylevel of level i; a level whose diagonal block vanishes
        at any site has a vanishing cell transfer and is solved like an empty one."""
        blocks = [self.blk[s].get((i, i)) for s in range(self.n)]
        if all(b is not None and _is_identity_block(b[1]) for b in blocks):
            return "identity"
        return "diag" if all(b is not None for b in blocks) else "empty"

    def _zero(self, kind, D, ni):
        return DeviceTensor.from_numpy(self.ctx, kind, np.zeros((D, ni, D), self.dtype))

    def recalculate(self, psi, tol=1e-12, krylovdim=30, maxiter=200):
        ctx, n, prec = self.ctx, self.n, self.precision
        lv, nlev = self.lv, self.nlev
        AL, AR, C = psi.AL, psi.AR, psi.C
        Dleft = [AL[s].dims[0] for s in range(n)]    # bond left of site s
        Dright = [AR[s].dims[2] for s in range(n)]   # bond right of site s
        eye = lambda D: DeviceTensor.from_numpy(ctx, L.GB_KIND_BOND, np.eye(D, dtype=self.dtype))
        prevL, prevR = self.GLl, self.GRl
        # GL[s][i]: level i of the left environment of site s
        GL = [[None] * nlev for _ in range(n)]
        GL[0][0] = DeviceTensor.from_numpy(
            ctx, L.GB_KIND_GL, np.eye(Dleft[0], dtype=self.dtype)[:, None, :])

        def left_cycle(i):
            # GL[s+1][i] = sum_{j <= i} GL[s][j] T(AL[s], W[s][j, i]), s = 0..n-1
            for s in range(n):
                acc = self._zero(L.GB_KIND_GL, Dright[s], lv[s + 1][i][1])
                for j in range(i + 1):
                    b = self.blk[s].get((j, i))
                    if b is not None and GL[s][j] is not None:
                        acc.axpy_(1.0, _transfer("L", ctx, GL[s][j], b[0], AL[s], prec))
                GL[(s + 1) % n][i] = acc

        if n > 1:
            left_cycle(0)
        rho_r = mul_tail(_as_mps(C[n - 1]), _adj(C[n - 1]))
        rho_r = _as_bond_t(rho_r)
        kd = min(Dleft[0] ** 2, krylovdim)
        for i in range(1, nlev):
            ni = lv[0][i][1]
            x0 = prevL[0][i] if prevL is not None else self._zero(L.GB_KIND_GL, Dleft[0], ni)
            GL[0][i] = self._zero(L.GB_KIND_GL, Dleft[0], ni)
            left_cycle(i)
            b = GL[0][i]
            kind = self._kind(i)
            diag = [self.blk[s].get((i, i)) for s in range(n)]

            def cell_T(v, reg):
                for s in range(n):
                    v = _transfer("L", ctx, v, diag[s][0], AL[s], prec)
                return _regularize(ctx, v, rho_r, eye(Dleft[0])) if reg else v

            if kind == "identity":
                x, _ = _gmres(lambda v: cell_T(v, True), b, x0, kd, maxiter, tol)
                GL[0][i] = x
                if n > 1:
                    left_cycle(i)
                for s in range(n):
                    r = _as_bond_t(mul_tail(_as_mps(C[s - 1]), _adj(C[s - 1])))
                    _regularize(ctx, GL[s][i], r, eye(Dleft[s]))
            else:
                if kind == "diag":
                    x, _ = _gmres(lambda v: cell_T(v, False), b, x0, kd, maxiter, tol)
                    GL[0][i] = x
                if n > 1:
                    left_cycle(i)

        # GR[s][i]: level i of the right environment of site s
        last = nlev - 1
        GR = [[None] * nlev for _ in range(n)]
        GR[n - 1][last] = DeviceTensor.from_numpy(
            ctx, L.GB_KIND_GR, np.eye(Dright[n - 1], dtype=self.dtype)[:, None, :])

        def right_cycle(i):
            # GR[s-1][i] = sum_{j >= i} T(AR[s], W[s][i, j]) GR[s][j], s = n-1..0
            for s in range(n - 1, -1, -1):
                acc = self._zero(L.GB_KIND_GR, Dleft[s], lv[s][i][1])
                for j in range(i, nlev):
                    b = self.blk[s].get((i, j))
                    if b is not None and GR[s][j] is not None:
                        acc.axpy_(1.0, _transfer("R", ctx, GR[s][j], b[0], AR[s], prec))
                GR[(s - 1) % n][i] = acc

        if n > 1:
            right_cycle(last)
        l_rr = _as_bond_t(mul_tail(_as_mps(_adj(C[n - 1])), C[n - 1]))
        kd = min(Dright[n - 1] ** 2, krylovdim)
        for i in range(nlev - 2, -1, -1):
            ni = lv[n][i][1]
            x0 = (prevR[n - 1][i] if prevR is not None
                  else self._zero(L.GB_KIND_GR, Dright[n - 1], ni))
            GR[n - 1][i] = self._zero(L.GB_KIND_GR, Dright[n - 1], ni)
            right_cycle(i)
            b = GR[n - 1][i]
            kind = self._kind(i)
            diag = [self.blk[s].get((i, i)) for s in range(n)]

            def cell_T(v, reg):
                for s in range(n - 1, -1, -1):
                    v = _transfer("R", ctx, v, diag[s][0], AR[s], prec)
                return _regularize(ctx, v, l_rr, eye(Dright[n - 1])) if reg else v

            if kind == "identity":
                x, _ = _gmres(lambda v: cell_T(v, True), b, x0, kd, maxiter, tol)
                GR[n - 1][i] = x
                if n > 1:
                    right_cycle(i)
                for s in range(n):
                    l = _as_bond_t(mul_tail(_as_mps(_adj(C[s])), C[s]))
                    _regularize(ctx, GR[s][i], l, eye(Dright[s]))
            else:
                if kind == "diag":
                    x, _ = _gmres(lambda v: cell_T(v, False), b, x0, kd, maxiter, tol)
                    GR[n - 1][i] = x
                if n > 1:
                    right_cycle(i)

        self.GLl, self.GRl = GL, GR
        self.GL, self.GR = [], []
        for s in range(n):
            wl = sum(k for _, k in lv[s])
            wr = sum(k for _, k in lv[s + 1])
            gl = DeviceTensor(ctx, L.GB_KIND_GL, self.dtype, (Dleft[s], wl, Dleft[s]))
            gr = DeviceTensor(ctx, L.GB_KIND_GR, self.dtype, (Dright[s], wr, Dright[s]))
            for i in range(nlev):
                L.check(L.lib().gb_env_channel_copy(ctx.handle, gl.handle, lv[s][i][0],
                                                    GL[s][i].handle, 0, lv[s][i][1]))
                L.check(L.lib().gb_env_channel_copy(ctx.handle, gr.handle, lv[s + 1][i][0],
                                                    GR[s][i].handle, 0, lv[s + 1][i][1]))
            self.GL.append(gl)
            self.GR.append(gr)
        return self


def _adj(C):
    from .infinite import adjoint
    return adjoint(C)


def _as_bond_t(A):
    from .infinite import _as_bond
    return _as_bond(A)


def _heff_ac(envs, s, backend):
    W = envs.H.device(envs.ctx, envs.dtype)[s]
    return DerivativeOperator(envs.ctx, L.GB_HEFF_AC, envs.GL[s], W, None, envs.GR[s], backend)


def _heff_c(envs, s, backend):
    return DerivativeOperator(envs.ctx, L.GB_HEFF_C, envs.GL[(s + 1) % envs.n], None, None,
                              envs.GR[s], backend)


def energy(psi, envs):
    """expectation_value(::InfiniteMPS, ::InfiniteMPOHamiltonian): the energy of one cell,
    sum over s of <AC[s]| GL[s] . W[s][:, :, :, end] . GR[s][end] |AC[s]> (expval.jl:150-161)."""
    ctx = envs.ctx
    total = 0.0
    for s in range(envs.n):
        W = envs.H.W[s]
        Wl = DeviceTensor.from_numpy(ctx, L.GB_KIND_MPO, np.ascontiguousarray(W[:, :, :, -1:]),
                                     envs.dtype)
        D = envs.GR[s].dims[0]
        GRl = DeviceTensor(ctx, L.GB_KIND_GR, envs.dtype, (D, 1, D))
        L.check(L.lib().gb_env_channel_copy(ctx.handle, GRl.handle, 0, envs.GR[s].handle,
                                            envs.GR[s].dims[1] - 1, 1))
        op = DerivativeOperator(ctx, L.GB_HEFF_AC, envs.GL[s], Wl, None, GRl, GB300Backend())
        ac = psi.AC(s)
        total += float(np.real(ac.dot(op(ac))))
    return total


def galerkin(psi, envs, backend=None):
    """calc_galerkin over the cell: the largest |(1 - AL AL') normalize(H_AC(AC))|."""
    worst = 0.0
    for s in range(envs.n):
        y = _heff_ac(envs, s, backend or GB300Backend())(psi.AC(s))
        y.normalize_()
        project_complement_(y, psi.AL[s])
        worst = max(worst, y.norm())
    return worst


def find_groundstate_vumps(psi, H, alg, envs=None):
    """find_groundstate(::InfiniteMPS, H, VUMPS()) for a cell.  Returns (psi, envs, eps,
    history) with the energy per site in the history."""
    n = len(psi)
    envs = envs or InfiniteEnvironmentsCell(psi, H, alg.backend.code)
    it = 0
    envs.recalculate(psi, tol=1e-10)
    eps = galerkin(psi, envs, alg.backend)
    envs.recalculate(psi, tol=_dyn_tol(eps, it, 1e-4))
    hist = []
    while True:
        solver = Lanczos(krylovdim=30, maxiter=200, tol=_dyn_tol(eps, it, 1e-3), eager=True)
        ALs = []
        for s in range(n):
            _, AC, _ = fixedpoint(_heff_ac(envs, s, alg.backend), psi.AC(s), "SR", solver)
            _, C, _ = fixedpoint(_heff_c(envs, s, alg.backend), psi.C[s], "SR", solver)
            ALs.append(regauge(AC, C))
        AR, Cs = uniform_rightorth(ALs, psi.C[n - 1], tol=_dyn_tol(eps, it, 1e-6))
        psi = InfiniteMPSCell(ALs, AR, Cs)
        envs.recalculate(psi, tol=_dyn_tol(eps, it, 1e-4))
        eps = galerkin(psi, envs, alg.backend)
        it += 1
        hist.append({"iter": it, "energy": energy(psi, envs) / n, "eps": eps})
        if eps <= alg.tol or it >= alg.maxiter:
            break
    return psi, envs, eps, hist


def timestep(psi, H, t, dt, alg=None, envs=None, imaginary_evolution=False, tolgauge=1e-14):
    """timestep(::InfiniteMPS, H, t, dt, TDVP()) for a cell (tdvp.jl:72-133,
    leftorthflag = true): every AC[s] and C[s] integrated with the same environments,
    AL[s] = regauge(AC[s], C[s]), the state rebuilt as InfiniteMPS(AL, C[end]) by the cell's
    uniform right gauge and the environments recalculated.  Returns (psi, envs)."""
    from .algorithms import TDVP
    from .derivatives import integrate
    from .infinite import regauge as _regauge
    alg = alg or TDVP()
    if psi.dtype.kind != "c" and not imaginary_evolution:
        raise TypeError("real-time evolution needs a complex InfiniteMPS")
    if envs is None:
        envs = InfiniteEnvironmentsCell(psi, H, alg.backend.code)
    if envs.GL is None:
        envs.recalculate(psi)
    n = len(psi)
    AL = []
    for s in range(n):
        AC = integrate(_heff_ac(envs, s, alg.backend), psi.AC(s), t, dt, alg.integrator,
                       imaginary_evolution)
        C = integrate(_heff_c(envs, s, alg.backend), psi.C[s], t, dt, alg.integrator,
                      imaginary_evolution)
        AL.append(_regauge(AC, C))
    AR, C = uniform_rightorth(AL, psi.C[n - 1], tol=tolgauge)
    psi = InfiniteMPSCell(AL, AR, C)
    envs.recalculate(psi)
    return psi, envs


def find_groundstate_idmrg(psi, H, alg, envs=None):
    """find_groundstate(::InfiniteMPS, H, IDMRG()) for a cell of n >= 1 sites
    (idmrg.jl:85-229): per site from left to right an AC eigensolve (started from the stored
    AC), the positive QR AC = AL[s] C[s] and GL[s+1] <- GL[s] T(AL[s]); then from right to
    left an AC eigensolve, the positive LQ AC = C[s-1] AR[s] and GR[s-1] <- T(AR[s]) GR[s]
    (un-normalised transfers, infinite_envs.jl:359-369).  The error is the change of the
    boundary bond tensor C[n-1]; the result is InfiniteMPS(AR) with recalculated
    environments.  Returns (psi, envs, eps, history), history entries carrying the energy
    change (E - E_old) / 2."""
    n = len(psi)
    ctx = psi.ctx
    envs = envs or InfiniteEnvironmentsCell(psi, H, alg.backend.code)
    envs.recalculate(psi, tol=1e-10)
    eps = galerkin(psi, envs, alg.backend)
    E_old = energy(psi, envs)
    Wd = H.device(ctx, envs.dtype)
    prec = envs.precision
    AL, AR, C = list(psi.AL), list(psi.AR), list(psi.C)
    AC = [psi.AC(s) for s in range(n)]
    GL, GR = list(envs.GL), list(envs.GR)

    def eig(pos, solver):
        h = DerivativeOperator(ctx, L.GB_HEFF_AC, GL[pos], Wd[pos], None, GR[pos], alg.backend)
        val, x, _ = fixedpoint(h, AC[pos], "SR", solver)
        return val, x

    it = 0
    hist = []
    while True:
        solver = Lanczos(krylovdim=30, maxiter=200, tol=_dyn_tol(eps, it, 1e-3), eager=True)
        C_old = C[n - 1]
        for pos in range(n):
            _, AC[pos] = eig(pos, solver)
            AL[pos], C[pos] = left_orth(AC[pos])
            GL[(pos + 1) % n] = _transfer("L", ctx, GL[pos], Wd[pos], AL[pos], prec)
        for pos in range(n - 1, -1, -1):
            E, AC[pos] = eig(pos, solver)
            C[pos - 1], AR[pos] = right_orth(AC[pos])
            GR[pos - 1] = _transfer("R", ctx, GR[pos], Wd[pos], AR[pos], prec)
        eps = _diff_norm(C[n - 1], C_old)
        it += 1
        hist.append({"iter": it, "energy_change": (E - E_old) / 2, "eps": eps})
        E_old = E
        if eps <= alg.tol or it >= alg.maxiter:
            break
    psi = InfiniteMPSCell.from_tensors(AR, tol=_dyn_tol(eps, it, 1e-6), maxiter=200)
    envs = InfiniteEnvironmentsCell(psi, H, alg.backend.code)
    envs.recalculate(psi, tol=1e-10)
    return psi, envs, eps, hist


class IDMRG2:
    """IDMRG2 defaults (idmrg.jl:46-71): tol 1e-10, maxiter 200, DynamicTol eigensolver;
    trunc = truncrank(maxdim) & trunctol(atol = cutoff)."""

    def __init__(self, maxdim, cutoff=1e-10, tol=1e-10, maxiter=200, backend=None):
        self.maxdim, self.cutoff = maxdim, cutoff
        self.tol, self.maxiter = tol, maxiter
        self.backend = backend or GB300Backend()


def _inv_bond(C):
    """C^-1 of a square bond tensor on the device: C = U S V' (cuSOLVER gesvd), C^-1 =
    V S^-1 U'.  Only the singular values cross to the host (to form S^-1)."""
    from .grassmann import _bond_as_mps, _diag, _mps_as_bond, _svd
    from .infinite import adjoint
    n = C.dims[0]
    if C.dims[1] != n:
        raise ValueError("inverse of a non-square bond tensor")
    U, s, Vh = _svd(_bond_as_mps(C), (n, 1, n))
    if s.size < n or not s[-1] > 0.0:
        raise np.linalg.LinAlgError("bond tensor is singular")
    V = _bond_as_mps(adjoint(Vh))
    return _mps_as_bond(mul_tail(mul_tail(V, _diag(C.ctx, 1.0 / s, C.dtype)),
                                 adjoint(_mps_as_bond(U))))


def find_groundstate_idmrg2(psi, H, alg, envs=None):
    """find_groundstate(::InfiniteMPS, H, IDMRG2(; trunc)) for a cell of n >= 2 sites
    (idmrg.jl:143-338): left-to-right two-site updates, the edge update across the cell
    boundary, right-to-left updates and the second edge update, each followed by
    un-normalised environment transfers (transfer_leftenv!/transfer_rightenv!,
    infinite_envs.jl:359-369); the error is the change of the boundary bond tensor.  The
    result is InfiniteMPS(AR) with recalculated environments.  Returns (psi, envs, eps,
    history); history entries carry the reference's energy change (the energy of a cell)."""
    n = len(psi)
    if n < 2:
        raise ValueError("unit cell should be >= 2")
    ctx = psi.ctx
    envs = envs or InfiniteEnvironmentsCell(psi, H, alg.backend.code)
    envs.recalculate(psi, tol=1e-10)
    eps = galerkin(psi, envs, alg.backend)
    E_old = energy(psi, envs)
    Wd = H.device(ctx, envs.dtype)
    prec = envs.precision
    AL, AR, C = list(psi.AL), list(psi.AR), list(psi.C)
    AC = [mul_tail(AL[i], C[i]) for i in range(n)]
    GL, GR = list(envs.GL), list(envs.GR)

    def eig2(pos, x0, solver):
        h = DerivativeOperator(ctx, L.GB_HEFF_AC2, GL[pos], Wd[pos], Wd[(pos + 1) % n],
                               GR[(pos + 1) % n], alg.backend)
        val, x, _ = fixedpoint(h, x0, "SR", solver)
        return val, x

    def split(x):
        al, c, ar, _ = svd_trunc(x, alg.maxdim, alg.cutoff, normalize=True)
        return al, c, ar

    tl = lambda pos: _transfer("L", ctx, GL[pos], Wd[pos], AL[pos], prec)
    tr = lambda pos: _transfer("R", ctx, GR[pos], Wd[pos], AR[pos], prec)
    it = 0
    hist = []
    while True:
        solver = Lanczos(krylovdim=30, maxiter=200, tol=_dyn_tol(eps, it, 1e-3), eager=True)
        for pos in range(n - 1):
            _, x = eig2(pos, ac2_from(AC[pos], AR[pos + 1]), solver)
            AL[pos], C[pos], AR[pos + 1] = split(x)
            AC[pos + 1] = mul_front(C[pos], AR[pos + 1])
            GL[pos + 1] = tl(pos)
            GR[pos] = tr(pos + 1)
        # the edge: bond between the last and the first site
        AL[n - 1] = mul_tail(AC[n - 1], _inv_bond(C[n - 1]))
        AC[0] = mul_tail(AL[0], C[0])
        _, x = eig2(n - 1, ac2_from(AL[n - 1], AC[0]), solver)
        al, c, ar = split(x)
        AL[n - 1], C[n - 1], AR[0] = al, c, ar
        AC[n - 1] = mul_tail(al, c)
        AC[0] = mul_front(c, ar)
        AL[0] = mul_tail(AC[0], _inv_bond(C[0]))
        C_old = c
        GL[0] = tl(n - 1)
        GR[n - 1] = tr(0)
        for pos in range(n - 2, -1, -1):
            _, x = eig2(pos, ac2_from(AL[pos], AC[pos + 1]), solver)
            al, c, ar = split(x)
            AL[pos], C[pos], AR[pos + 1] = al, c, ar
            AC[pos] = mul_tail(al, c)
            AC[pos + 1] = mul_front(c, ar)
            GL[pos + 1] = tl(pos)
            GR[pos] = tr(pos + 1)
        # the edge again
        AC[n - 1] = mul_front(C[n - 2], AR[n - 1])
        AR[0] = mul_front(_inv_bond(C[n - 1]), AC[0])
        E, x = eig2(n - 1, ac2_from(AC[n - 1], AR[0]), solver)
        al, c, ar = split(x)
        AL[n - 1], C[n - 1], AR[0] = al, c, ar
        AR[n - 1] = mul_front(_inv_bond(C[n - 2]), mul_tail(al, c))
        AC[0] = mul_front(c, ar)
        GL[0] = tl(n - 1)
        GR[n - 1] = tr(0)
        Cn, Co = C[n - 1].numpy(), C_old.numpy()
        k = min(Cn.shape[0], Co.shape[0])
        eps = float(np.linalg.norm(Cn[:k, :k] - Co[:k, :k]))
        dE = (E - E_old) / 2
        if n == 2:
            dE /= 2
        E_old = E
        it += 1
        hist.append({"iter": it, "energy_change": dE, "eps": eps})
        if eps <= alg.tol or it >= alg.maxiter:
            break
    psi = InfiniteMPSCell.from_tensors(AR, tol=_dyn_tol(eps, it, 1e-6), maxiter=200)
    envs = InfiniteEnvironmentsCell(psi, H, alg.backend.code)
    envs.recalculate(psi, tol=1e-10)
    return psi, envs, eps, hist
