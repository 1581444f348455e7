"""Krylov eigensolver / exponentiator (oracle restatement of KrylovKit as MPSKit uses it).

MPSKit calls `KrylovKit.eigsolve(A, x0, 1, :SR, Lanczos(...))` through `fixedpoint`
(src/algorithms/fixedpoint.jl:15-18) and `KrylovKit.exponentiate` through `integrate`
(src/algorithms/timestep/integrators.jl:21-30).  KrylovKit is not vendored; this module
restates its published Lanczos algorithm:

  * the factorisation starts from x0/|x0| (one matvec), every expansion is one matvec,
    with full re-orthogonalisation of the new vector against the basis;
  * the projected (Rayleigh-quotient) matrix is diagonalised when the subspace is full,
    when beta <= tol, or -- with `eager` -- after every expansion; a Ritz pair is
    converged when |beta * U[K, i]| <= tol (absolute tolerance on the residual norm);
  * when the subspace reaches `krylovdim` and is not converged, it is shrunk to
    keep = (3*krylovdim + 2*howmany) // 5 Ritz vectors plus the residual direction
    (thick restart), at most `maxiter` times.

`Info` mirrors KrylovKit's ConvergenceInfo fields that MPSKit reads
(`converged`, `normres`, `numops`, `numiter`; dmrg.jl:153, 239).
"""
import numpy as np


class Info:
    def __init__(self, converged, normres, numops, numiter):
        self.converged = converged
        self.normres = normres
        self.numops = numops
        self.numiter = numiter

    def __repr__(self):
        return (f"Info(converged={self.converged}, normres={self.normres:.3e}, "
                f"numops={self.numops}, numiter={self.numiter})")


def _dot(a, b):
    return np.vdot(a.ravel(), b.ravel())


def lanczos_eigsolve(A, x0, krylovdim=30, maxiter=100, tol=1e-12, eager=False, which="SR"):
    """Lowest (SR) eigenpair of the hermitian map A.  Returns (val, vec, info)."""
    assert which == "SR"
    howmany = 1
    shape = x0.shape
    n = x0.size
    dt = np.result_type(x0.dtype, np.float64)
    V = np.zeros((krylovdim + 1, n), dtype=dt)
    x = x0.ravel().astype(dt)
    V[0] = x / np.linalg.norm(x)
    H = np.zeros((krylovdim + 1, krylovdim + 1))
    numops = 0
    numiter = 1
    K = 0            # current basis size (number of orthonormal vectors with A applied)
    r = None
    beta = 0.0
    while True:
        # expand: apply A to V[K]
        w = A(V[K].reshape(shape)).ravel().astype(dt)
        numops += 1
        # full orthogonalisation (two passes, classical Gram-Schmidt)
        c = V[:K + 1].conj() @ w
        w = w - V[:K + 1].T @ c
        c2 = V[:K + 1].conj() @ w
        w = w - V[:K + 1].T @ c2
        h = (c + c2)
        H[:K + 1, K] = h.real
        H[K, :K + 1] = h.real
        K += 1
        beta = np.linalg.norm(w)
        r = w
        if K == krylovdim or beta <= tol or (eager and K >= howmany):
            D, U = np.linalg.eigh(H[:K, :K])
            f = beta * U[K - 1, :]
            converged = 0
            while converged < K and abs(f[converged]) <= tol:
                converged += 1
            if converged >= howmany or beta <= tol:
                break
        if K < krylovdim:
            V[K] = r / beta
            continue
        if numiter == maxiter:
            break
        # thick restart
        keep = (3 * krylovdim + 2 * howmany) // 5
        Vk = U[:, :keep].T @ V[:K]
        V[:keep] = Vk
        H[:] = 0.0
        H[np.arange(keep), np.arange(keep)] = D[:keep]
        # the arrow couples the kept Ritz vectors to the residual direction
        H[keep, :keep] = f[:keep]
        H[:keep, keep] = f[:keep]
        V[keep] = r / beta
        K = keep
        # next matvec applies A to V[keep]; the arrow already in H[:keep, keep]
        numiter += 1
        # special expand that accounts for the arrow: handled by the generic code since
        # H[:K+1, K] is overwritten by the projections c (which reproduce the arrow).
    vec = (U[:, 0] @ V[:K]).reshape(shape)
    vec = vec / np.linalg.norm(vec)
    normres = abs(f[0])
    info = Info(int(converged), float(normres), numops, numiter)
    return float(D[0]), vec, info


def lanczos_exponentiate(A, t, x0, krylovdim=30, maxiter=100, tol=1e-12):
    """y = exp(t*A) x0 for hermitian A and complex scalar t, via Lanczos with
    time-step subdivision (KrylovKit `exponentiate`, restated).  Returns (y, info)."""
    shape = x0.shape
    y = x0.ravel().astype(np.complex128)
    total = complex(t)
    tau_left = 1.0            # remaining fraction of t
    numops = 0
    numiter = 0
    tau = 1.0
    while tau_left > 0 and numiter < maxiter * 50:
        numiter += 1
        nrm = np.linalg.norm(y)
        if nrm == 0:
            break
        V = [y / nrm]
        alphas, betas = [], []
        K = 0
        happy = False
        for j in range(krylovdim):
            w = A(V[j].reshape(shape)).ravel().astype(np.complex128)
            numops += 1
            a = np.vdot(V[j], w).real
            w = w - a * V[j] - (betas[-1] * V[j - 1] if j > 0 else 0)
            Vm = np.array(V)
            w = w - Vm.T @ (Vm.conj() @ w)
            b = np.linalg.norm(w)
            alphas.append(a)
            K = j + 1
            if b <= tol * 1e-3:
                happy = True
                betas.append(b)
                break
            betas.append(b)
            V.append(w / b)
        T = np.diag(alphas) + np.diag(betas[:K - 1], 1) + np.diag(betas[:K - 1], -1)
        ev, U = np.linalg.eigh(T)
        tau = min(tau, tau_left)
        while True:
            e1 = U[0, :].conj()
            c = U @ (np.exp(total * tau * ev) * e1)
            # error estimate: size of the coefficient along the next Krylov vector
            err = abs(betas[K - 1] * c[K - 1]) * nrm if not happy else 0.0
            if err <= tol * tau or tau < 1e-12:
                break
            tau *= 0.5
        Vm = np.array(V[:K])
        y = nrm * (c @ Vm)
        tau_left -= tau
        if tau_left < 1e-15:
            tau_left = 0.0
        tau = min(2 * tau, 1.0)
    info = Info(int(tau_left == 0.0), 0.0, numops, numiter)
    return y.reshape(shape), info


def gmres_solve(A, b, x0, krylovdim=30, maxiter=100, tol=1e-12, a0=0.0, a1=1.0):
    """Solve (a0 + a1*A) x = b by restarted GMRES (KrylovKit `linsolve` with GMRES).
    Returns (x, info)."""
    shape = b.shape
    bb = b.ravel().astype(np.complex128)
    x = x0.ravel().astype(np.complex128)

    def op(v):
        return a0 * v + a1 * A(v.reshape(shape)).ravel()

    numops = 0
    for it in range(maxiter):
        r = bb - op(x)
        numops += 1
        beta = np.linalg.norm(r)
        if beta <= tol:
            return x.reshape(shape), Info(1, float(beta), numops, it)
        V = [r / beta]
        Hm = np.zeros((krylovdim + 1, krylovdim), dtype=np.complex128)
        k = 0
        for j in range(krylovdim):
            w = op(V[j])
            numops += 1
            for i in range(j + 1):
                Hm[i, j] = np.vdot(V[i], w)
                w = w - Hm[i, j] * V[i]
            for i in range(j + 1):
                c = np.vdot(V[i], w)
                Hm[i, j] += c
                w = w - c * V[i]
            Hm[j + 1, j] = np.linalg.norm(w)
            k = j + 1
            e = np.zeros(k + 1, dtype=np.complex128)
            e[0] = beta
            yls = np.linalg.lstsq(Hm[:k + 1, :k], e, rcond=None)[0]
            res = np.linalg.norm(e - Hm[:k + 1, :k] @ yls)
            if res <= tol or Hm[j + 1, j].real < 1e-300:
                break
            V.append(w / Hm[j + 1, j])
        x = x + np.array(V[:k]).T @ yls
        if res <= tol:
            return x.reshape(shape), Info(1, float(res), numops, it + 1)
    r = bb - op(x)
    return x.reshape(shape), Info(0, float(np.linalg.norm(r)), numops + 1, maxiter)
