"""VUMPS on a one-site unit cell with InfiniteMPOHamiltonian environments (oracle).

Restates:
  * uniform_leftorth! / uniform_rightorth! (positive QR / LQ iterations)
        -- src/states/ortho.jl:210-340
  * regauge!(AC, C) = Q_AC Q_C'                -- src/states/ortho.jl:178-184
  * initialize_environments / compute_leftenvs! / compute_rightenvs! for an
    InfiniteMPOHamiltonian: level by level, linsolve(flip(T), b, prev, GMRES, 1, -1)
    with the regularised transfer matrix on identity levels
        -- src/environments/infinite_envs.jl:177-346, src/transfermatrix/transfermatrix.jl:189-237
  * VUMPS dominant_eigsolve / localupdate / gauge / envs steps
        -- src/algorithms/groundstate/vumps.jl:62-192
  * DynamicTol adaptation of the eigensolver, environment and gauge tolerances
        -- src/utility/dynamictols.jl:86-89, src/utility/defaults.jl:22-93
  * expectation_value(InfiniteMPS, InfiniteMPOHamiltonian) -- src/algorithms/expval.jl:150-161
  * l_LL = 1, r_LL = C C', l_RR = C' C, r_RR = 1 -- src/states/infinitemps.jl:349-408
  * timestep(::InfiniteMPS, H, t, dt, TDVP()) for a one-site cell -- integrate AC and C with
    the same environments, regauge, uniform gauge, recalculate
        -- src/algorithms/timestep/tdvp.jl:72-133
  * find_groundstate(::InfiniteMPS, H, IDMRG()) for a one-site cell -- left and right
    eigensolve of AC with positive QR / LQ and un-normalised environment transfers, the
    change of C as the error, InfiniteMPS(AR) and recalculated environments at the end
        -- src/algorithms/groundstate/idmrg.jl:85-216, src/environments/infinite_envs.jl:359-369

The Arnoldi acceleration of the gauge iterations (after eig_miniter = 10 steps) is not
restated; the QR/LQ iterations converge to the same fixed point.
"""
import numpy as np

from . import derivatives as dv
from .krylov import gmres_solve, lanczos_eigsolve, lanczos_exponentiate
from .mps import lq_pos, qr_pos


def dyn_tol(eps, it, factor, tmin=1e-14, tmax=1e-4):
    """DynamicTol (dynamictols.jl:86-89) with the Defaults bounds."""
    return min(max(factor * eps / np.sqrt(max(it, 1)), tmin), tmax)


def levels(chans):
    off = np.concatenate([[0], np.cumsum(chans)]).astype(int)
    return [slice(off[i], off[i + 1]) for i in range(len(chans))]


class InfiniteMPS1:
    """One-site unit cell: AL, AR, C, AC with AL C = C AR = AC."""

    def __init__(self, AL, AR, C):
        self.AL, self.AR, self.C = AL, AR, C

    @property
    def AC(self):
        return np.einsum("asb,bc->asc", self.AL, self.C)


def uniform_leftorth(A, C0, tol=1e-14, maxiter=200):
    D, d, _ = A.shape
    C = C0 / np.linalg.norm(C0)
    for it in range(maxiter):
        CA = np.einsum("ab,bsc->asc", C, A)
        Q, R = qr_pos(CA.reshape(D * d, D, order="F"))
        AL = Q.reshape(D, d, D, order="F")
        Cn = R / np.linalg.norm(R)
        err = np.linalg.norm(C - Cn)
        C = Cn
        if err < tol:
            break
    return AL, C


def uniform_rightorth(A, C0, tol=1e-14, maxiter=200):
    D, d, _ = A.shape
    C = C0 / np.linalg.norm(C0)
    for it in range(maxiter):
        AC = np.einsum("asb,bc->asc", A, C)
        Lm, Q = lq_pos(AC.reshape(D, d * D, order="F"))
        AR = Q.reshape(D, d, D, order="F")
        Cn = Lm / np.linalg.norm(Lm)
        err = np.linalg.norm(C - Cn)
        C = Cn
        if err < tol:
            break
    return AR, C


def infinite_mps(A, tol=1e-14):
    """InfiniteMPS(A) with mixed-canonical gauge fixing (order :LR)."""
    D = A.shape[0]
    AL, C = uniform_leftorth(A, np.eye(D, dtype=A.dtype), tol)
    AR, C = uniform_rightorth(AL, C, tol)
    return InfiniteMPS1(AL, AR, C)


def regauge(AC, C):
    """regauge!(AC, C) -> AL = Q_AC Q_C' (ortho.jl:178-184)."""
    D, d, Dr = AC.shape
    Qac, _ = qr_pos(AC.reshape(D * d, Dr, order="F"))
    Qc, _ = qr_pos(C)
    return (Qac @ Qc.conj().T).reshape(D, d, Dr, order="F")


def _is_identity_block(B):
    n, d = B.shape[0], B.shape[1]
    ref = np.einsum("ab,st->astb", np.eye(n), np.eye(d))
    return B.shape == ref.shape and np.allclose(B, ref, atol=0)


def infinite_envs(psi, W, chans, GL0=None, GR0=None, tol=1e-12, krylovdim=30, maxiter=200):
    """compute_leftenvs! / compute_rightenvs! for a one-site cell (infinite_envs.jl:207-346).
    Returns GL[a, w, a'], GR[b', w, b] over the full channel space."""
    AL, AR, C = psi.AL, psi.AR, psi.C
    D = AL.shape[0]
    dt = np.result_type(AL.dtype, W.dtype)
    lv = levels(chans)
    n = len(lv)
    w = sum(chans)
    kd = min(D * D, krylovdim)
    # left: GL = (1, 0, 0)
    GL = np.zeros((D, w, D), dtype=dt)
    GL[:, lv[0], :] = np.eye(D)[:, None, :]
    l_LL = np.eye(D, dtype=dt)
    r_LL = C @ C.conj().T
    for i in range(1, n):
        prev = (GL0[:, lv[i], :] if GL0 is not None else np.zeros((D, chans[i], D), dtype=dt))
        b = np.zeros((D, chans[i], D), dtype=dt)
        for j in range(i):
            blk = W[lv[j], :, :, lv[i]]
            if np.any(blk != 0):
                b += dv.transfer_left(GL[:, lv[j], :], blk, AL, AL)
        diag = W[lv[i], :, :, lv[i]]
        if i == n - 1 or _is_identity_block(diag):
            def op(x):
                y = dv.transfer_left(x, diag, AL, AL)
                lam = np.einsum("xy,ywx->w", r_LL, y)
                return y - lam[None, :, None] * l_LL[:, None, :]
            x, _ = gmres_solve(op, b, prev, krylovdim=kd, maxiter=maxiter, tol=tol, a0=1.0, a1=-1.0)
            lam = np.einsum("xy,ywx->w", r_LL, x)
            x = x - lam[None, :, None] * l_LL[:, None, :]
        elif np.any(diag != 0):
            op = lambda x: dv.transfer_left(x, diag, AL, AL)
            x, _ = gmres_solve(op, b, prev, krylovdim=kd, maxiter=maxiter, tol=tol, a0=1.0, a1=-1.0)
        else:
            x = b
        GL[:, lv[i], :] = x
    # right: GR = (0, 0, 1)^T
    GR = np.zeros((D, w, D), dtype=dt)
    GR[:, lv[n - 1], :] = np.eye(D)[:, None, :]
    l_RR = C.conj().T @ C
    r_RR = np.eye(D, dtype=dt)
    for i in range(n - 2, -1, -1):
        prev = (GR0[:, lv[i], :] if GR0 is not None else np.zeros((D, chans[i], D), dtype=dt))
        b = np.zeros((D, chans[i], D), dtype=dt)
        for j in range(i + 1, n):
            blk = W[lv[i], :, :, lv[j]]
            if np.any(blk != 0):
                b += dv.transfer_right(GR[:, lv[j], :], blk, AR, AR)
        diag = W[lv[i], :, :, lv[i]]
        if i == 0 or _is_identity_block(diag):
            def op(x):
                y = dv.transfer_right(x, diag, AR, AR)
                lam = np.einsum("xy,ywx->w", l_RR, y)
                return y - lam[None, :, None] * r_RR[:, None, :]
            x, _ = gmres_solve(op, b, prev, krylovdim=kd, maxiter=maxiter, tol=tol, a0=1.0, a1=-1.0)
            lam = np.einsum("xy,ywx->w", l_RR, x)
            x = x - lam[None, :, None] * r_RR[:, None, :]
        elif np.any(diag != 0):
            op = lambda x: dv.transfer_right(x, diag, AR, AR)
            x, _ = gmres_solve(op, b, prev, krylovdim=kd, maxiter=maxiter, tol=tol, a0=1.0, a1=-1.0)
        else:
            x = b
        GR[:, lv[i], :] = x
    return GL, GR


def energy_density(psi, W, GL, GR):
    """expectation_value(::InfiniteMPS, ::InfiniteMPOHamiltonian) (expval.jl:150-161):
    contract_mpo_expval(AC, GL, H[:, 1, 1, end], GR[end])."""
    return dv.contract_mpo_expval(psi.AC, GL, W[:, :, :, -1:], GR[:, -1:, :]).real


def galerkin(psi, W, GL, GR):
    """calc_galerkin (toolbox.jl:63-70) for the single site of the cell."""
    AC = psi.AC
    y = dv.JordanAC(GL, W, GR)(AC)
    y = y / np.linalg.norm(y)
    D, d, Dr = AC.shape
    A = psi.AL.reshape(D * d, Dr, order="F")
    Y = y.reshape(D * d, Dr, order="F")
    return float(np.linalg.norm(Y - A @ (A.conj().T @ Y)))


def vumps(psi, H, tol=1e-10, maxiter=200, verbose=False):
    """find_groundstate(::InfiniteMPS, H, VUMPS()) for a one-site cell.
    Returns (psi, GL, GR, eps, history)."""
    W = H[0]
    chans = H.chans[0]
    it = 0
    GL, GR = infinite_envs(psi, W, chans, tol=1e-10)
    eps = galerkin(psi, W, GL, GR)
    GL, GR = infinite_envs(psi, W, chans, GL, GR, tol=dyn_tol(eps, it, 1e-4))
    hist = []
    while True:
        et = dyn_tol(eps, it, 1e-3)
        _, AC, _ = lanczos_eigsolve(dv.JordanAC(GL, W, GR), psi.AC, krylovdim=30, maxiter=200,
                                    tol=et, eager=True)
        _, C, _ = lanczos_eigsolve(dv.CHam(GL, GR), psi.C, krylovdim=30, maxiter=200, tol=et,
                                   eager=True)
        AL = regauge(AC, C)
        AR, C = uniform_rightorth(AL, psi.C, tol=dyn_tol(eps, it, 1e-6))
        psi = InfiniteMPS1(AL, AR, C)
        GL, GR = infinite_envs(psi, W, chans, GL, GR, tol=dyn_tol(eps, it, 1e-4))
        eps = galerkin(psi, W, GL, GR)
        it += 1
        e = energy_density(psi, W, GL, GR)
        hist.append((it, e, eps))
        if verbose:
            print(f"VUMPS {it}: e = {e:.14f} eps = {eps:.3e}")
        if eps <= tol or it >= maxiter:
            break
    return psi, GL, GR, eps, hist


def tdvp_timestep_infinite(psi, H, dt, GL=None, GR=None, imaginary=False, tol=1e-12):
    """One TDVP step of a one-site InfiniteMPS (tdvp.jl:91-133, leftorthflag = true):
    AC' = exp(-i dt H_AC) AC and C' = exp(-i dt H_C) C with the environments of psi
    (-dt instead of -i dt for imaginary time), AL = regauge(AC', C'), then the uniform
    right gauge from AL with the old C as starting point.  Returns (psi', GL, GR) with the
    environments of psi'."""
    W = H[0]
    chans = H.chans[0]
    if GL is None:
        GL, GR = infinite_envs(psi, W, chans, tol=tol)
    tt = -dt if imaginary else -1j * dt
    AC, _ = lanczos_exponentiate(dv.JordanAC(GL, W, GR), tt, psi.AC, krylovdim=30, tol=tol)
    C, _ = lanczos_exponentiate(dv.CHam(GL, GR), tt, psi.C.astype(np.complex128), krylovdim=30,
                                tol=tol)
    AL = regauge(AC, C)
    AR, C2 = uniform_rightorth(AL, psi.C, tol=1e-14)
    psi2 = InfiniteMPS1(AL, AR, C2)
    GL, GR = infinite_envs(psi2, W, chans, GL, GR, tol=tol)
    return psi2, GL, GR


def idmrg(psi, H, tol=1e-10, maxiter=200):
    """find_groundstate(::InfiniteMPS, H, IDMRG()) for a one-site cell.  Each iteration
    (idmrg.jl:194-228): AC eigensolve (:SR, DynamicTol factor 1e-3), AL C = AC (positive
    QR), GL <- GL T(AL) without normalisation (transfer_leftenv!, infinite_envs.jl:359-363);
    AC eigensolve from the previous AC, C AR = AC (positive LQ), GR <- T(AR) GR; the error
    is |C - C_old| (idmrg.jl:150-159).  The result is InfiniteMPS(AR) gauge-fixed with the
    DynamicTol gauge tolerance and recalculated environments (idmrg.jl:131-135).
    Returns (psi, GL, GR, eps, history) with history entries (iteration, dE, eps), dE the
    energy change per site (idmrg.jl:162)."""
    W = H[0]
    chans = H.chans[0]
    D, d, _ = psi.AL.shape
    GL, GR = infinite_envs(psi, W, chans, tol=1e-10)
    eps = galerkin(psi, W, GL, GR)
    E_old = energy_density(psi, W, GL, GR)
    AC, C = psi.AC, psi.C
    AR = psi.AR
    it = 0
    hist = []
    while True:
        et = dyn_tol(eps, it, 1e-3)
        C_old = C
        _, AC, _ = lanczos_eigsolve(dv.JordanAC(GL, W, GR), AC, krylovdim=30, maxiter=200,
                                    tol=et, eager=True)
        Q, C = qr_pos(AC.reshape(D * d, D, order="F"))
        AL = Q.reshape(D, d, D, order="F")
        GL = dv.transfer_left(GL, W, AL, AL)
        E, AC, _ = lanczos_eigsolve(dv.JordanAC(GL, W, GR), AC, krylovdim=30, maxiter=200,
                                    tol=et, eager=True)
        C, Q = lq_pos(AC.reshape(D, d * D, order="F"))
        AR = Q.reshape(D, d, D, order="F")
        GR = dv.transfer_right(GR, W, AR, AR)
        eps = float(np.linalg.norm(C - C_old))
        it += 1
        hist.append((it, (E - E_old) / 2, eps))
        E_old = E
        if eps <= tol or it >= maxiter:
            break
    D0 = AR.shape[0]
    gtol = dyn_tol(eps, it, 1e-6)
    AL2, C2 = uniform_leftorth(AR, np.eye(D0, dtype=AR.dtype), gtol)
    AR2, C2 = uniform_rightorth(AL2, C2, gtol)
    psi2 = InfiniteMPS1(AL2, AR2, C2)
    GL, GR = infinite_envs(psi2, W, chans, GL, GR, tol=1e-10)
    return psi2, GL, GR, eps, hist
