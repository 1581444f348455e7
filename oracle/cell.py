"""InfiniteMPS with a unit cell of L >= 1 sites: uniform gauge, InfiniteMPOHamiltonian
environments, VUMPS and IDMRG2 (oracle; test infrastructure only).

Restates, for a cell of L sites (0-based here; the reference counts sites from 1 and wraps
periodically):
  * uniform_leftorth! / uniform_rightorth! over the cell (positive QR / LQ sweeps, only the
    boundary bond tensor normalised)                         -- src/states/ortho.jl:214-340
  * InfiniteMPS(As) = left then right gauge fixing (order :LR)
  * compute_leftenvs! / compute_rightenvs! with left_cyclethrough! / right_cyclethrough!:
    level by level, the inhomogeneous term is the image of the zero-started level through
    the whole cell, the level is solved at the cell boundary with the product transfer
    matrix (regularised on identity levels), propagated through the cell again, and on
    identity levels every site's value has its fixed-point component removed
                                                   -- src/environments/infinite_envs.jl:207-346
  * expectation_value(InfiniteMPS, InfiniteMPOHamiltonian) = sum over the cell
                                                                 -- src/algorithms/expval.jl:150-161
  * calc_galerkin = the largest site error                       -- src/algorithms/toolbox.jl:63-79
  * VUMPS on the cell: per site AC and C eigensolves and regauge, then the uniform right
    gauge from the new AL and the old boundary C, then the environments
                                                   -- src/algorithms/groundstate/vumps.jl:101-192
  * IDMRG2: left-to-right two-site updates, the edge update across the cell boundary, the
    right-to-left updates and the second edge update, with un-normalised environment
    transfers; the error is the change of the boundary bond tensor
                                                   -- src/algorithms/groundstate/idmrg.jl:143-338
"""
import numpy as np

from . import derivatives as dv
from .krylov import gmres_solve, lanczos_eigsolve
from .mps import lq_pos, qr_pos, svd_trunc
from .vumps import _is_identity_block, dyn_tol, levels


class InfiniteMPSCell:
    """AL[i] C[i] = C[i-1] AR[i] = AC[i]; C[i] sits right of site i (C[-1] = C[L-1])."""

    def __init__(self, AL, AR, C):
        self.AL, self.AR, self.C = list(AL), list(AR), list(C)

    def __len__(self):
        return len(self.AL)

    def AC(self, i):
        return np.einsum("asb,bc->asc", self.AL[i], self.C[i])


def uniform_leftorth(As, C0, tol=1e-14, maxiter=200):
    """C[i-1] A[i] = AL[i] C[i] around the cell until the boundary C stops changing."""
    L = len(As)
    AL = [None] * L
    C = [None] * L
    C[L - 1] = C0 / np.linalg.norm(C0)
    for _ in range(maxiter):
        before = C[L - 1]
        for i in range(L):
            CA = np.einsum("ab,bsc->asc", C[i - 1], As[i])
            Dl, d, Dr = CA.shape
            Q, R = qr_pos(CA.reshape(Dl * d, Dr, order="F"))
            AL[i] = Q.reshape(Dl, d, Q.shape[1], order="F")
            C[i] = R
        C[L - 1] = C[L - 1] / np.linalg.norm(C[L - 1])
        if np.linalg.norm(before - C[L - 1]) < tol:
            break
    return AL, C


def uniform_rightorth(As, C0, tol=1e-14, maxiter=200):
    """A[i] C[i] = C[i-1] AR[i] from the last site to the first, until C[L-1] is stable."""
    L = len(As)
    AR = [None] * L
    C = [None] * L
    C[L - 1] = C0 / np.linalg.norm(C0)
    for _ in range(maxiter):
        before = C[L - 1]
        for i in range(L - 1, -1, -1):
            AC = np.einsum("asb,bc->asc", As[i], C[i])
            Dl, d, Dr = AC.shape
            Lm, Q = lq_pos(AC.reshape(Dl, d * Dr, order="F"))
            AR[i] = Q.reshape(Q.shape[0], d, Dr, order="F")
            C[i - 1] = Lm
        C[L - 1] = C[L - 1] / np.linalg.norm(C[L - 1])
        if np.linalg.norm(before - C[L - 1]) < tol:
            break
    return AR, C


def infinite_mps(As, tol=1e-14, maxiter=200):
    """InfiniteMPS(As) with order :LR."""
    D = As[0].shape[0]
    AL, C = uniform_leftorth(As, np.eye(D, dtype=As[0].dtype), tol, maxiter)
    AR, C = uniform_rightorth(AL, C[-1], tol, maxiter)
    return InfiniteMPSCell(AL, AR, C)


def _level_kind(H, i):
    """'identity' if every site's diagonal block of level i is the identity, 'diag' if any
    is nonzero, 'empty' otherwise (isidentitylevel / isemptylevel)."""
    L = len(H.W)
    blocks = []
    for s in range(L):
        ll, lr = levels(H.chans[s]), levels(H.chans[s + 1])
        blocks.append(H.W[s][ll[i], :, :, lr[i]])
    if all(b.shape[0] == b.shape[3] and _is_identity_block(b) for b in blocks):
        return "identity", blocks
    if any(np.any(b != 0) for b in blocks):
        return "diag", blocks
    return "empty", blocks


def infinite_envs(psi, H, GL0=None, GR0=None, tol=1e-12, krylovdim=30, maxiter=200):
    """compute_leftenvs! / compute_rightenvs! for a cell.  GL[s] is the left environment of
    site s (on the bond left of it), GR[s] the right one (on the bond right of it); both over
    the full channel space of their MPO bond, layout GL[a, w, a'], GR[b', w, b]."""
    L = len(psi)
    AL, AR, C = psi.AL, psi.AR, psi.C
    dt = np.result_type(AL[0].dtype, H.W[0].dtype)
    nlev = len(H.chans[0])
    lvl = [levels(H.chans[s]) for s in range(L + 1)]   # levels of the bond left of site s
    Dbond = [AL[s].shape[0] for s in range(L)]          # dimension of the bond left of site s
    GL = [np.zeros((Dbond[s], sum(H.chans[s]), Dbond[s]), dtype=dt) for s in range(L)]
    GR = [np.zeros((Dbond[(s + 1) % L], sum(H.chans[s + 1]), Dbond[(s + 1) % L]), dtype=dt)
          for s in range(L)]

    # ---------------- left
    GL[0][:, lvl[0][0], :] = np.eye(Dbond[0])[:, None, :]

    def left_cycle(i):
        # GL[s+1][i] = sum_{j <= i} GL[s][j] T(AL[s], W[s][j, i]) around the cell
        for s in range(L):
            Dn = AL[s].shape[2]
            acc = np.zeros((Dn, H.chans[s + 1][i], Dn), dtype=dt)
            for j in range(i + 1):
                blk = H.W[s][lvl[s][j], :, :, lvl[s + 1][i]]
                if np.any(blk != 0):
                    acc += dv.transfer_left(GL[s][:, lvl[s][j], :], blk, AL[s], AL[s])
            GL[(s + 1) % L][:, lvl[(s + 1) % L][i], :] = acc

    if L > 1:
        left_cycle(0)
    rho_r = C[L - 1] @ C[L - 1].conj().T     # r_LL at the cell boundary
    eye0 = np.eye(Dbond[0], dtype=dt)
    for i in range(1, nlev):
        prev = (GL0[0][:, lvl[0][i], :] if GL0 is not None
                else np.zeros((Dbond[0], H.chans[0][i], Dbond[0]), dtype=dt))
        GL[0][:, lvl[0][i], :] = 0
        left_cycle(i)
        b = GL[0][:, lvl[0][i], :].copy()
        kind, diag = _level_kind(H, i)
        kd = min(Dbond[0] ** 2, krylovdim)

        def cell_T(x):
            for s in range(L):
                x = dv.transfer_left(x, diag[s], AL[s], AL[s])
            return x

        if kind == "identity":
            def op(x):
                y = cell_T(x)
                lam = np.einsum("xy,ywx->w", rho_r, y)
                return y - lam[None, :, None] * eye0[:, None, :]
            x, _ = gmres_solve(op, b, prev, krylovdim=kd, maxiter=maxiter, tol=tol, a0=1.0,
                               a1=-1.0)
            GL[0][:, lvl[0][i], :] = x
            if L > 1:
                left_cycle(i)
            for s in range(L):
                r = C[s - 1] @ C[s - 1].conj().T
                g = GL[s][:, lvl[s][i], :]
                lam = np.einsum("xy,ywx->w", r, g)
                GL[s][:, lvl[s][i], :] = g - lam[None, :, None] * np.eye(Dbond[s])[:, None, :]
        else:
            if kind == "diag":
                x, _ = gmres_solve(cell_T, b, prev, krylovdim=kd, maxiter=maxiter, tol=tol,
                                   a0=1.0, a1=-1.0)
                GL[0][:, lvl[0][i], :] = x
            if L > 1:
                left_cycle(i)

    # ---------------- right
    last = nlev - 1
    DL = [AR[s].shape[2] for s in range(L)]             # dimension of the bond right of site s
    GR[L - 1][:, lvl[L][last], :] = np.eye(DL[L - 1])[:, None, :]

    def right_cycle(i):
        # GR[s-1][i] = sum_{j >= i} T(AR[s], W[s][i, j]) GR[s][j], s = L-1 .. 0
        for s in range(L - 1, -1, -1):
            Dn = AR[s].shape[0]
            acc = np.zeros((Dn, H.chans[s][i], Dn), dtype=dt)
            for j in range(i, nlev):
                blk = H.W[s][lvl[s][i], :, :, lvl[s + 1][j]]
                if np.any(blk != 0):
                    acc += dv.transfer_right(GR[s][:, lvl[s + 1][j], :], blk, AR[s], AR[s])
            GR[(s - 1) % L][:, lvl[s][i], :] = acc

    if L > 1:
        right_cycle(last)
    rho_l = C[L - 1].conj().T @ C[L - 1]     # l_RR at the cell boundary
    eyeL = np.eye(DL[L - 1], dtype=dt)
    for i in range(nlev - 2, -1, -1):
        prev = (GR0[L - 1][:, lvl[L][i], :] if GR0 is not None
                else np.zeros((DL[L - 1], H.chans[L][i], DL[L - 1]), dtype=dt))
        GR[L - 1][:, lvl[L][i], :] = 0
        right_cycle(i)
        b = GR[L - 1][:, lvl[L][i], :].copy()
        kind, diag = _level_kind(H, i)
        kd = min(DL[L - 1] ** 2, krylovdim)

        def cell_T(x):
            for s in range(L - 1, -1, -1):
                x = dv.transfer_right(x, diag[s], AR[s], AR[s])
            return x

        if kind == "identity":
            def op(x):
                y = cell_T(x)
                lam = np.einsum("xy,ywx->w", rho_l, y)
                return y - lam[None, :, None] * eyeL[:, None, :]
            x, _ = gmres_solve(op, b, prev, krylovdim=kd, maxiter=maxiter, tol=tol, a0=1.0,
                               a1=-1.0)
            GR[L - 1][:, lvl[L][i], :] = x
            if L > 1:
                right_cycle(i)
            for s in range(L):
                l = C[s].conj().T @ C[s]
                g = GR[s][:, lvl[s + 1][i], :]
                lam = np.einsum("xy,ywx->w", l, g)
                GR[s][:, lvl[s + 1][i], :] = g - lam[None, :, None] * np.eye(DL[s])[:, None, :]
        else:
            if kind == "diag":
                x, _ = gmres_solve(cell_T, b, prev, krylovdim=kd, maxiter=maxiter, tol=tol,
                                   a0=1.0, a1=-1.0)
                GR[L - 1][:, lvl[L][i], :] = x
            if L > 1:
                right_cycle(i)
    return GL, GR


def energy(psi, H, GL, GR):
    """expectation_value: the energy of one unit cell (sum over its sites)."""
    e = 0.0
    for s in range(len(psi)):
        e += dv.contract_mpo_expval(psi.AC(s), GL[s], H.W[s][:, :, :, -1:],
                                    GR[s][:, -1:, :]).real
    return float(e)


def galerkin(psi, H, GL, GR):
    """calc_galerkin: max over the cell of |(1 - AL AL') normalize(H_AC(AC))|."""
    worst = 0.0
    for s in range(len(psi)):
        AC = psi.AC(s)
        y = dv.JordanAC(GL[s], H.W[s], GR[s])(AC)
        y = y / np.linalg.norm(y)
        D, d, Dr = AC.shape
        A = psi.AL[s].reshape(D * d, Dr, order="F")
        Y = y.reshape(D * d, Dr, order="F")
        worst = max(worst, float(np.linalg.norm(Y - A @ (A.conj().T @ Y))))
    return worst


def _regauge(AC, C):
    D, d, Dr = AC.shape
    Qac, _ = qr_pos(AC.reshape(D * d, Dr, order="F"))
    Qc, _ = qr_pos(C)
    return (Qac @ Qc.conj().T).reshape(D, d, Dr, order="F")


def vumps(psi, H, tol=1e-10, maxiter=200):
    """find_groundstate(::InfiniteMPS, H, VUMPS()) for a cell.  Returns (psi, GL, GR, eps,
    history) with history entries (iteration, energy per site, eps)."""
    L = len(psi)
    it = 0
    GL, GR = infinite_envs(psi, H, tol=1e-10)
    eps = galerkin(psi, H, GL, GR)
    GL, GR = infinite_envs(psi, H, GL, GR, tol=dyn_tol(eps, it, 1e-4))
    hist = []
    while True:
        et = dyn_tol(eps, it, 1e-3)
        ALs = []
        for s in range(L):
            _, AC, _ = lanczos_eigsolve(dv.JordanAC(GL[s], H.W[s], GR[s]), psi.AC(s),
                                        krylovdim=30, maxiter=200, tol=et, eager=True)
            _, C, _ = lanczos_eigsolve(dv.CHam(GL[(s + 1) % L], GR[s]), psi.C[s],
                                       krylovdim=30, maxiter=200, tol=et, eager=True)
            ALs.append(_regauge(AC, C))
        AR, Cs = uniform_rightorth(ALs, psi.C[L - 1], tol=dyn_tol(eps, it, 1e-6))
        psi = InfiniteMPSCell(ALs, AR, Cs)
        GL, GR = infinite_envs(psi, H, GL, GR, tol=dyn_tol(eps, it, 1e-4))
        eps = galerkin(psi, H, GL, GR)
        it += 1
        hist.append((it, energy(psi, H, GL, GR) / L, eps))
        if eps <= tol or it >= maxiter:
            break
    return psi, GL, GR, eps, hist


def _ac2(A, B):
    """AC2[l s1; r s2] = A[l s1; m] B[m s2; r]."""
    return np.einsum("asm,mtb->asbt", A, B)


def _split(ac2, maxdim, atol):
    """svd_trunc! of AC2 -> (al, c, ar) with c normalised (diagonal)."""
    Dl, d1, Dr, d2 = ac2.shape
    U, S, Vh, _ = svd_trunc(ac2.reshape(Dl * d1, Dr * d2, order="F"), maxdim, atol)
    S = S / np.linalg.norm(S)
    k = S.size
    al = U.reshape(Dl, d1, k, order="F")
    ar = np.transpose(Vh.reshape(k, Dr, d2, order="F"), (0, 2, 1))
    return al, np.diag(S).astype(ac2.dtype), ar


def _eig_ac2(GL, W1, W2, GR, x0, tol):
    val, x, _ = lanczos_eigsolve(dv.JordanAC2(GL, W1, W2, GR), x0, krylovdim=30, maxiter=200,
                                 tol=tol, eager=True)
    return val, x


def _c_change(C, C_old):
    """|C - C_old| on the common leading block (isometries onto the smaller space)."""
    k = min(C.shape[0], C_old.shape[0])
    return float(np.linalg.norm(C[:k, :k] - C_old[:k, :k]))


def idmrg2(psi, H, maxdim, atol=1e-10, tol=1e-10, maxiter=200):
    """find_groundstate(::InfiniteMPS, H, IDMRG2(; trunc)) for a cell of L >= 2 sites
    (idmrg.jl:143-338; trunc = truncrank(maxdim) & trunctol(atol)).  Returns (psi, GL, GR,
    eps, history) with history entries (iteration, dE, eps); dE is the reference's energy
    change (E - E_old) / 2, halved once more for L = 2 (idmrg.jl:161-162) -- the energy of
    one unit cell."""
    L = len(psi)
    if L < 2:
        raise ValueError("unit cell should be >= 2")
    Ws = H.W
    GL, GR = infinite_envs(psi, H, tol=1e-10)
    eps = galerkin(psi, H, GL, GR)
    E_old = energy(psi, H, GL, GR)
    AL, AR, C = list(psi.AL), list(psi.AR), list(psi.C)
    AC = [np.einsum("asb,bc->asc", AL[i], C[i]) for i in range(L)]
    tl = lambda G, s: dv.transfer_left(G, Ws[s], AL[s], AL[s])
    tr = lambda G, s: dv.transfer_right(G, Ws[s], AR[s], AR[s])
    inv = np.linalg.inv
    it = 0
    hist = []
    while True:
        et = dyn_tol(eps, it, 1e-3)
        # left to right
        for pos in range(L - 1):
            _, x = _eig_ac2(GL[pos], Ws[pos], Ws[pos + 1], GR[pos + 1],
                            _ac2(AC[pos], AR[pos + 1]), et)
            al, c, ar = _split(x, maxdim, atol)
            AL[pos], C[pos], AR[pos + 1] = al, c, ar
            AC[pos + 1] = np.einsum("ab,bsc->asc", c, ar)
            GL[pos + 1] = tl(GL[pos], pos)
            GR[pos] = tr(GR[pos + 1], pos + 1)
        # the edge (bond between the last and the first site)
        AL[L - 1] = np.einsum("asb,bc->asc", AC[L - 1], inv(C[L - 1]))
        AC[0] = np.einsum("asb,bc->asc", AL[0], C[0])
        _, x = _eig_ac2(GL[L - 1], Ws[L - 1], Ws[0], GR[0], _ac2(AL[L - 1], AC[0]), et)
        al, c, ar = _split(x, maxdim, atol)
        AL[L - 1], C[L - 1], AR[0] = al, c, ar
        AC[L - 1] = np.einsum("asb,bc->asc", al, c)
        AC[0] = np.einsum("ab,bsc->asc", c, ar)
        AL[0] = np.einsum("asb,bc->asc", AC[0], inv(C[0]))
        C_old = c
        GL[0] = tl(GL[L - 1], L - 1)
        GR[L - 1] = tr(GR[0], 0)
        # right to left
        for pos in range(L - 2, -1, -1):
            _, x = _eig_ac2(GL[pos], Ws[pos], Ws[pos + 1], GR[pos + 1],
                            _ac2(AL[pos], AC[pos + 1]), et)
            al, c, ar = _split(x, maxdim, atol)
            AL[pos], C[pos], AR[pos + 1] = al, c, ar
            AC[pos] = np.einsum("asb,bc->asc", al, c)
            AC[pos + 1] = np.einsum("ab,bsc->asc", c, ar)
            GL[pos + 1] = tl(GL[pos], pos)
            GR[pos] = tr(GR[pos + 1], pos + 1)
        # the edge again
        AC[L - 1] = np.einsum("ab,bsc->asc", C[L - 2], AR[L - 1])
        AR[0] = np.einsum("ab,bsc->asc", inv(C[L - 1]), AC[0])
        E, x = _eig_ac2(GL[L - 1], Ws[L - 1], Ws[0], GR[0], _ac2(AC[L - 1], AR[0]), et)
        al, c, ar = _split(x, maxdim, atol)
        AL[L - 1], C[L - 1], AR[0] = al, c, ar
        AR[L - 1] = np.einsum("ab,bsc->asc", inv(C[L - 2]), np.einsum("asb,bc->asc", al, c))
        AC[0] = np.einsum("ab,bsc->asc", c, ar)
        GL[0] = tl(GL[L - 1], L - 1)
        GR[L - 1] = tr(GR[0], 0)
        eps = _c_change(C[L - 1], C_old)
        dE = (E - E_old) / 2
        if L == 2:
            dE /= 2
        E_old = E
        it += 1
        hist.append((it, float(np.real(dE)), eps))
        if eps <= tol or it >= maxiter:
            break
    gtol = dyn_tol(eps, it, 1e-6)
    D0 = AR[0].shape[0]
    ALn, Cn = uniform_leftorth(AR, np.eye(D0, dtype=AR[0].dtype), gtol)
    ARn, Cn = uniform_rightorth(ALn, Cn[-1], gtol)
    psi = InfiniteMPSCell(ALn, ARn, Cn)
    GL, GR = infinite_envs(psi, H, tol=1e-10)
    return psi, GL, GR, eps, hist


def idmrg1(psi, H, tol=1e-10, maxiter=200):
    """find_groundstate(::InfiniteMPS, H, IDMRG()) for a cell of L >= 1 sites
    (idmrg.jl:85-229): per site from left to right an AC eigensolve (started from the stored
    AC), the positive QR AC = AL C and GL[s+1] <- GL[s] T(AL[s]); then per site from right to
    left an AC eigensolve, the positive LQ AC = C[s-1] AR[s] and GR[s-1] <- T(AR[s]) GR[s]
    (un-normalised transfers, infinite_envs.jl:359-369).  The error is the change of the
    boundary bond tensor C[L-1]; dE = (E - E_old) / 2.  The result is InfiniteMPS(AR).
    Returns (psi, GL, GR, eps, history) with history entries (iteration, dE, eps)."""
    L = len(psi)
    Ws = H.W
    GL, GR = infinite_envs(psi, H, tol=1e-10)
    eps = galerkin(psi, H, GL, GR)
    E_old = energy(psi, H, GL, GR)
    AL, AR, C = list(psi.AL), list(psi.AR), list(psi.C)
    AC = [psi.AC(s) for s in range(L)]
    it = 0
    hist = []
    while True:
        et = dyn_tol(eps, it, 1e-3)
        C_old = C[L - 1]
        for pos in range(L):
            _, AC[pos], _ = lanczos_eigsolve(dv.JordanAC(GL[pos], Ws[pos], GR[pos]), AC[pos],
                                             krylovdim=30, maxiter=200, tol=et, eager=True)
            Dl, d, Dr = AC[pos].shape
            Q, R = qr_pos(AC[pos].reshape(Dl * d, Dr, order="F"))
            AL[pos], C[pos] = Q.reshape(Dl, d, Q.shape[1], order="F"), R
            GL[(pos + 1) % L] = dv.transfer_left(GL[pos], Ws[pos], AL[pos], AL[pos])
        for pos in range(L - 1, -1, -1):
            E, AC[pos], _ = lanczos_eigsolve(dv.JordanAC(GL[pos], Ws[pos], GR[pos]), AC[pos],
                                             krylovdim=30, maxiter=200, tol=et, eager=True)
            Dl, d, Dr = AC[pos].shape
            Lm, Q = lq_pos(AC[pos].reshape(Dl, d * Dr, order="F"))
            AR[pos], C[pos - 1] = Q.reshape(Q.shape[0], d, Dr, order="F"), Lm
            GR[pos - 1] = dv.transfer_right(GR[pos], Ws[pos], AR[pos], AR[pos])
        eps = _c_change(C[L - 1], C_old)
        it += 1
        hist.append((it, float(np.real(E - E_old)) / 2, eps))
        E_old = E
        if eps <= tol or it >= maxiter:
            break
    gtol = dyn_tol(eps, it, 1e-6)
    D0 = AR[0].shape[0]
    ALn, Cn = uniform_leftorth(AR, np.eye(D0, dtype=AR[0].dtype), gtol)
    ARn, Cn = uniform_rightorth(ALn, Cn[-1], gtol)
    psi = InfiniteMPSCell(ALn, ARn, Cn)
    GL, GR = infinite_envs(psi, H, tol=1e-10)
    return psi, GL, GR, eps, hist


def tdvp_timestep(psi, H, dt, GL=None, GR=None, imaginary=False, tol=1e-12):
    """One TDVP step of an InfiniteMPS cell (tdvp.jl:91-133, leftorthflag = true): per site
    AC'[s] = exp(-i dt H_AC[s]) AC[s] and C'[s] = exp(-i dt H_C[s]) C[s] with the
    environments of psi (-dt for imaginary time), AL[s] = regauge(AC'[s], C'[s]), then
    InfiniteMPS(AL, C[end]) -- the cell's uniform right gauge.  Returns (psi', GL, GR) with
    the environments of psi'."""
    from .krylov import lanczos_exponentiate
    from .vumps import regauge
    L = len(psi)
    if GL is None:
        GL, GR = infinite_envs(psi, H, tol=tol)
    tt = -dt if imaginary else -1j * dt
    AL = []
    for s in range(L):
        AC, _ = lanczos_exponentiate(dv.JordanAC(GL[s], H.W[s], GR[s]), tt, psi.AC(s),
                                     krylovdim=30, tol=tol)
        C, _ = lanczos_exponentiate(dv.CHam(GL[(s + 1) % L], GR[s]), tt,
                                    psi.C[s].astype(np.complex128), krylovdim=30, tol=tol)
        AL.append(regauge(AC, C))
    AR, C2 = uniform_rightorth(AL, psi.C[-1], tol=1e-14)
    psi2 = InfiniteMPSCell(AL, AR, C2)
    GL, GR = infinite_envs(psi2, H, tol=tol)
    return psi2, GL, GR
