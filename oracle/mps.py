"""Finite MPS containers, gauge steps and the DMRG / DMRG2 drivers (oracle).

Restates:
  * FiniteMPS(f, elt, P, maxV) random constructor + QR normalisation sweep
      -- src/states/finitemps.jl:229-282 (positive QR at :234-237)
  * AC2(psi, site; kind)                    -- src/states/finitemps.jl:376-385
  * left_gauge / right_gauge / gauge2!      -- src/states/orthoview.jl:322-420
  * project_complement!                     -- src/utility/utility.jl:22
  * calc_galerkin                           -- src/algorithms/toolbox.jl:63-70
  * adapt_solver(::AdaptiveKrylov)          -- src/utility/dynamictols.jl:182-235
  * DMRG / DMRG2 local_update! and sweep    -- src/algorithms/groundstate/dmrg.jl:121-354
  * FiniteEnvironments leftenv / rightenv   -- src/environments/finite_envs.jl:31-49, 110-151
  * expectation_value(FiniteMPS, H)         -- src/algorithms/expval.jl:136-141

Sites are 0-based.  C[b] is the bond matrix between site b-1 and site b
(C[0], C[L] are the 1x1 boundaries).  GL[i] is the left environment of site i,
GR[i] the right environment of site i.
"""
import numpy as np

from . import derivatives as dv
from .krylov import lanczos_eigsolve


# ---------------------------------------------------------------- factorisations

def qr_pos(M):
    """QR with non-negative diagonal of R (MatrixAlgebraKit Householder(positive=true))."""
    Q, R = np.linalg.qr(M)
    s = np.sign(np.diag(R).real)
    s[s == 0] = 1
    # for complex diagonal, rotate the phase to the positive real axis
    ph = np.diag(R) / np.where(np.abs(np.diag(R)) > 0, np.abs(np.diag(R)), 1)
    ph[np.abs(np.diag(R)) == 0] = 1
    Q = Q * ph[None, :]
    R = R * ph.conj()[:, None]
    return Q, R


def lq_pos(M):
    """LQ with non-negative diagonal of L."""
    Q, R = qr_pos(M.conj().T)
    return R.conj().T, Q.conj().T


def svd_trunc(M, maxdim=None, atol=0.0):
    """svd_trunc with truncrank(maxdim) & trunctol(atol=atol).  Returns U, S, Vh, eps
    where eps is the 2-norm of the discarded singular values."""
    U, S, Vh = np.linalg.svd(M, full_matrices=False)
    keep = int(np.sum(S > atol))
    if maxdim is not None:
        keep = min(keep, maxdim)
    keep = max(keep, 1)
    eps = float(np.linalg.norm(S[keep:]))
    return U[:, :keep], S[:keep], Vh[:keep], eps


# ---------------------------------------------------------------- FiniteMPS

class FiniteMPS:
    """AL/AR/C storage with an explicit centre bond: AL[i] is valid for i < center,
    AR[i] for i >= center, C[center] is the current centre matrix."""

    def __init__(self, AL, AR, C, center=0, qb=None, qp=None):
        self.AL = AL
        self.AR = AR
        self.C = C
        self.center = center
        # U(1): charges of every bond (qb[b] between sites b-1 and b) and of the physical leg
        self.qb = qb
        self.qp = qp

    def __len__(self):
        return len(self.AL)

    def copy(self):
        cp = lambda xs: [None if x is None else x.copy() for x in xs]
        return FiniteMPS(cp(self.AL), cp(self.AR), cp(self.C), self.center,
                         None if self.qb is None else cp(self.qb), self.qp)

    def ac(self, i):
        """The centre-site tensor AC[i] for a centre bond at i or i+1 (or an explicitly
        stored AC, as `psi.AC[i] = ...` leaves it in the reference)."""
        if getattr(self, "ac_site", None) == i:
            return self.ac_tensor
        if self.center == i:
            return self.AC(i)
        if self.center == i + 1:
            return self.ACL(i)
        raise ValueError(f"site {i} is not adjacent to the centre bond {self.center}")

    def al(self, i):
        """AL[i]; computed from AC[i] by a positive QR when the centre bond is i
        (the reference computes it lazily the same way)."""
        if i < self.center:
            return self.AL[i]
        ac = self.ac(i)
        Dl, d, Dr = ac.shape
        if self.qb is not None:
            from .u1 import fuse, left_orth_u1
            Q, _, _ = left_orth_u1(ac.reshape(Dl * d, Dr, order="F"), fuse(self.qb[i], self.qp),
                                   self.qb[i + 1])
        else:
            Q, _ = qr_pos(ac.reshape(Dl * d, Dr, order="F"))
        return Q.reshape(Dl, d, Q.shape[1], order="F")

    def AC(self, i):
        """AC[i] = C[i] * AR[i] (valid when the centre bond is i)."""
        return np.einsum("ab,bsc->asc", self.C[i], self.AR[i])

    def ACL(self, i):
        """AC[i] = AL[i] * C[i+1] (valid when the centre bond is i+1)."""
        return np.einsum("asb,bc->asc", self.AL[i], self.C[i + 1])

    @property
    def dtype(self):
        return self.AL[0].dtype


def bond_dims(L, d, D):
    """Virtual dims limited to full rank (finitemps.jl:257-274)."""
    V = [1] * (L + 1)
    for k in range(1, L):
        V[k] = min(V[k - 1] * d, D)
    for k in range(L - 1, 0, -1):
        V[k] = min(V[k], V[k + 1] * d)
    return V


def random_initial_tensors(L, d, D, seed, dtype=np.complex128):
    """Seeded i.i.d. normal entries (re, im ~ N(0,1) for complex) on the full-rank
    virtual spaces -- the synthetic stand-in for `FiniteMPS(randn, elt, ...)`."""
    rng = np.random.default_rng(seed)
    V = bond_dims(L, d, D)
    As = []
    for i in range(L):
        shape = (V[i], d, V[i + 1])
        if np.dtype(dtype).kind == "c":
            a = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
        else:
            a = rng.standard_normal(shape)
        # store in Fortran (column-major) order like TensorKit; values are order-agnostic
        As.append(np.asarray(a, dtype=dtype))
    return As


def finite_mps_from_tensors(As, normalize=True, charges=None):
    """FiniteMPS(As; normalize) (finitemps.jl:229-250): positive-QR sweep left->right,
    then an LQ sweep right->left to build the AR gauge (what the reference does lazily
    on first access of `psi.AR`).  `charges` = (bond charges, physical charges) gives a
    U(1)-symmetric state whose factorisations act per charge block (oracle.u1)."""
    from .u1 import fuse, left_orth_u1
    L = len(As)
    As = [a.copy() for a in As]
    AL = [None] * L
    C = [None] * (L + 1)
    qb = qp = None
    if charges is not None:
        qb = [np.asarray(q, np.int32) for q in charges[0]]
        qp = np.asarray(charges[1], np.int32)
    for i in range(L):
        Dl, d, Dr = As[i].shape
        M = As[i].reshape(Dl * d, Dr, order="F")
        if qb is not None:
            Q, R, qb[i + 1] = left_orth_u1(M, fuse(qb[i], qp), qb[i + 1])
        else:
            Q, R = qr_pos(M)
        AL[i] = Q.reshape(Dl, d, Q.shape[1], order="F")
        if normalize:
            R = R / np.linalg.norm(R)
        if i < L - 1:
            As[i + 1] = np.einsum("ab,bsc->asc", R, As[i + 1])
    C[L] = R
    psi = FiniteMPS(AL, [None] * L, C, center=L, qb=qb, qp=qp)
    right_canonicalize(psi)
    return psi


def _col_charges(qp, qr):
    """Charges of the fused column (s, r) of A[l; s r]: q[s + d*r] = q_r - q_s."""
    return (np.asarray(qr)[None, :] - np.asarray(qp)[:, None]).reshape(-1, order="F")


def right_canonicalize(psi):
    """Build AR[i] and C[i] from the centre at bond L by positive LQ moves."""
    from .u1 import right_orth_u1
    L = len(psi)
    X = psi.C[L]
    for i in range(L - 1, -1, -1):
        A = np.einsum("asb,bc->asc", psi.AL[i], X)
        Dl, d, Dr = A.shape
        M = A.reshape(Dl, d * Dr, order="F")
        if psi.qb is not None:
            Lm, Q, qk = right_orth_u1(M, psi.qb[i], _col_charges(psi.qp, psi.qb[i + 1]))
            assert np.array_equal(qk, psi.qb[i]), "LQ sweep changed a bond space"
        else:
            Lm, Q = lq_pos(M)
        psi.AR[i] = Q.reshape(Q.shape[0], d, Dr, order="F")
        X = Lm
        psi.C[i] = Lm
    # C[0] is the 1x1 norm factor
    psi.center = 0
    return psi


# ---------------------------------------------------------------- environments

class FiniteEnvironments:
    """Lazy GL/GR cache keyed on object identity of AL/AR (finite_envs.jl:110-151)."""

    def __init__(self, psi, H):
        L = len(psi)
        dt = np.result_type(psi.dtype, H.dtype)
        self.H = H
        self.GL = [None] * (L + 1)
        self.GR = [None] * (L + 1)
        self.GL[0] = np.ones((1, 1, 1), dtype=dt)
        self.GR[L - 1] = np.ones((1, 1, 1), dtype=dt)
        self.ldep = [None] * L
        self.rdep = [None] * L

    def leftenv(self, i, psi):
        a = None
        for j in range(i):
            if psi.AL[j] is not self.ldep[j]:
                a = j
                break
        if a is not None:
            for j in range(a, i):
                self.GL[j + 1] = dv.transfer_left(self.GL[j], self.H[j], psi.AL[j], psi.AL[j])
                self.ldep[j] = psi.AL[j]
        return self.GL[i]

    def rightenv(self, i, psi):
        L = len(psi)
        a = None
        for j in range(L - 1, i, -1):
            if psi.AR[j] is not self.rdep[j]:
                a = j
                break
        if a is not None:
            for j in range(a, i, -1):
                self.GR[j - 1] = dv.transfer_right(self.GR[j], self.H[j], psi.AR[j], psi.AR[j])
                self.rdep[j] = psi.AR[j]
        return self.GR[i]


def AC2_hamiltonian(pos, psi, H, envs, prepare=True):
    return dv.JordanAC2(envs.leftenv(pos, psi), H[pos], H[pos + 1],
                        envs.rightenv(pos + 1, psi), prepare=prepare)


def AC_hamiltonian(pos, psi, H, envs, prepare=True):
    return dv.JordanAC(envs.leftenv(pos, psi), H[pos], envs.rightenv(pos, psi), prepare=prepare)


def expectation_value(psi, H, envs, site=0):
    """<psi|H|psi> / <psi|psi> evaluated at a site whose AC is current (expval.jl:136-141)."""
    AC = psi.ac(site)
    Heff = AC_hamiltonian(site, psi, H, envs)
    return np.vdot(AC, Heff(AC)).real / np.vdot(AC, AC).real


# ---------------------------------------------------------------- adaptive solver

class AdaptiveKrylov:
    """AdaptiveKrylov defaults (dynamictols.jl:182-194)."""

    def __init__(self, krylovdim_min=3, krylovdim_max=20, iter_min=1, iter_max=1,
                 tol_min=1e-12, tol_max=1e-2, truncation_factor=1e-1, tol_factor=1e-1,
                 eager=True):
        self.krylovdim_min = krylovdim_min
        self.krylovdim_max = krylovdim_max
        self.iter_min = iter_min
        self.iter_max = iter_max
        self.tol_min = tol_min
        self.tol_max = tol_max
        self.truncation_factor = truncation_factor
        self.tol_factor = tol_factor
        self.eager = eager

    def adapt(self, decay_rate=0.0, g_local=0.0, g_global=0.0, eps_trunc=0.0):
        """adapt_solver(::AdaptiveKrylov) (dynamictols.jl:204-235) -> (krylovdim, maxiter, tol)."""
        tol = min(max(max(self.truncation_factor * eps_trunc, self.tol_factor * g_global),
                      self.tol_min), self.tol_max)
        rho = min(max(decay_rate, 0.0), 1.0)
        if not (0 < rho < 1):
            if rho == 0:
                return self.krylovdim_min, self.iter_min, tol
            return self.krylovdim_max, self.iter_max, tol
        R = max(g_local, self.tol_min) / tol
        nmat = int(round(np.log(R) / np.log(1 / rho)))
        kd = min(max(nmat, self.krylovdim_min), self.krylovdim_max)
        cld = -((-5 * nmat) // (2 * kd))
        mi = min(max(cld - 3, self.iter_min), self.iter_max)
        return kd, mi, tol


# ---------------------------------------------------------------- DMRG2 / DMRG

class DMRG2:
    def __init__(self, maxdim, cutoff=0.0, tol=1e-10, maxiter=200, alg_eigsolve=None):
        self.maxdim = maxdim
        self.cutoff = cutoff
        self.tol = tol
        self.maxiter = maxiter
        self.alg_eigsolve = alg_eigsolve or AdaptiveKrylov()


class DMRG:
    def __init__(self, tol=1e-10, maxiter=200, alg_eigsolve=None, alg_gauge=None,
                 alg_expand=None):
        self.tol = tol
        self.maxiter = maxiter
        self.alg_eigsolve = alg_eigsolve or AdaptiveKrylov()
        # None: the positive QR/LQ gauge; a DMRG3S: the perturbed, truncated gauge
        self.alg_gauge = alg_gauge
        # None, or an OptimalExpand run ahead of every local update (dmrg.jl:128-134)
        self.alg_expand = alg_expand


class OptimalExpand:
    """OptimalExpand(; trunc = truncrank(add)) (changebonds/optimalexpand.jl:36-47): at
    most `add` directions are added to a bond per expansion."""

    def __init__(self, add):
        self.add = add


def _left_null(M):
    """Orthonormal basis of the complement of the column space of M (m x n, m >= n)."""
    Q, _ = np.linalg.qr(M, mode="complete")
    return Q[:, M.shape[1]:]


def _ac2_matrix(ac2):
    """AC2[l s1; r s2] as the matrix (l s1) x (s2 r)."""
    Dl, d1, Dr, d2 = ac2.shape
    return np.transpose(ac2, (0, 1, 3, 2)).reshape(Dl * d1, d2 * Dr, order="F")


def optimal_expand(pos, right, psi, H, envs, alg):
    """changebond!(site, dir, psi, H, ::OptimalExpand, envs) (optimalexpand.jl:122-187):
    the two-site update H_AC2 (AC2) projected onto the complements of the two sites
    (left_null / right_null), its `add` dominant directions appended to the bond -- with
    zero weight, so the state is unchanged -- and the sites regauged."""
    eps34 = np.finfo(np.float64).eps ** 0.75
    if right:
        left, rt = psi.ac(pos), psi.AR[pos + 1]
        Dl, d, Dr = left.shape
        Dn = rt.shape[2]
        lmat = left.reshape(Dl * d, Dr, order="F")
        RT = rt.reshape(Dr, d * Dn, order="F")
        NL = _left_null(lmat)
        NR = _left_null(RT.conj().T).conj().T
        ac2 = np.einsum("asm,mtb->asbt", left, rt)
        g2 = NL.conj().T @ _ac2_matrix(AC2_hamiltonian(pos, psi, H, envs)(ac2)) @ NR.conj().T
        nrm = np.linalg.norm(g2)
        if nrm <= eps34 or g2.size == 0:
            return
        _, _, Vh, _ = svd_trunc(g2 / nrm, alg.add, 0.0)
        k = Vh.shape[0]
        nal, nc = qr_pos(np.concatenate([lmat, np.zeros((Dl * d, k), dtype=lmat.dtype)], axis=1))
        nar = np.concatenate([RT, Vh @ NR], axis=0)
        psi.AL[pos] = nal.reshape(Dl, d, nal.shape[1], order="F")
        psi.C[pos + 1] = nc / np.linalg.norm(nc)
        psi.AR[pos + 1] = nar.reshape(Dr + k, d, Dn, order="F")
        psi.center = pos + 1
    else:
        lf, rgt = psi.AL[pos - 1], psi.ac(pos)
        Dp, d, Dl = lf.shape
        Dr = rgt.shape[2]
        lmat = lf.reshape(Dp * d, Dl, order="F")
        RT = rgt.reshape(Dl, d * Dr, order="F")
        NL = _left_null(lmat)
        NR = _left_null(RT.conj().T).conj().T
        ac2 = np.einsum("asm,mtb->asbt", lf, rgt)
        g2 = (NL.conj().T @ _ac2_matrix(AC2_hamiltonian(pos - 1, psi, H, envs)(ac2))
              @ NR.conj().T)
        nrm = np.linalg.norm(g2)
        if nrm <= eps34 or g2.size == 0:
            return
        U, _, _, _ = svd_trunc(g2 / nrm, alg.add, 0.0)
        k = U.shape[1]
        nc, Qr = lq_pos(np.concatenate([RT, np.zeros((k, d * Dr), dtype=RT.dtype)], axis=0))
        psi.AR[pos] = Qr.reshape(Qr.shape[0], d, Dr, order="F")
        psi.C[pos] = nc / np.linalg.norm(nc)
        psi.AL[pos - 1] = np.concatenate([lmat, NL @ U], axis=1).reshape(Dp, d, Dl + k,
                                                                          order="F")
        psi.center = pos


class SketchedExpand:
    """SketchedExpand(; trunc = truncrank(add), oversampling) (changebonds/sketchedexpand.jl:
    41-73).  The random isometries (randisometry) are drawn from numpy's PCG64 seeded with
    `seed`, one Gaussian matrix per expansion in call order (the reference draws from Julia's
    RNG, which cannot be reproduced here)."""

    def __init__(self, add, oversampling=0, seed=0):
        self.add, self.oversampling = add, oversampling
        self.rng = np.random.default_rng(seed)

    def gaussian(self, m, n, dtype):
        g = self.rng.standard_normal((m, n))
        if np.dtype(dtype).kind == "c":
            g = g + 1j * self.rng.standard_normal((m, n))
        return g.astype(dtype)

    def sketch(self, comp, other):
        """sketch_space: (l, k) = (sketch columns, target added directions) in the sketched
        complement `comp`.  Both are also capped by the other site's complement `other`:
        beyond it the orthonormalised directions cannot stay orthogonal to the state (the
        reference leaves them arbitrary)."""
        cap = min(comp, other)
        k = min(self.add, cap)
        return min(k + self.oversampling, cap), k

    def sketch_u1(self, comp, other):
        """sketch_space for a U(1) complement (charge -> dimension maps, capped by `other`):
        sample_space (randexpand.jl:160-165) draws a uniform weight per direction and keeps
        the `add` largest, giving per-sector counts k_c; the oversampling adds
        min(dim, oversampling) per sector, capped (infimum).  Returns (charges, l_c, k_c)."""
        qs = [c for c in sorted(comp) if min(comp[c], other.get(c, 0)) > 0]
        cap = np.array([min(comp[c], other[c]) for c in qs], dtype=np.int64)
        weights = self.rng.random(int(cap.sum()))
        owner = np.repeat(np.arange(len(qs)), cap)
        chosen = np.argsort(-weights, kind="stable")[:min(self.add, int(cap.sum()))]
        kc = np.array([np.sum(owner[chosen] == i) for i in range(len(qs))], dtype=np.int64)
        return np.asarray(qs, dtype=np.int32), np.minimum(cap, kc + self.oversampling), kc


def _u1_comp(q_fused, q_bond):
    """charge -> dimension of fused(...) minus the bond (the complement space, U(1))."""
    out = {}
    for c in np.asarray(q_fused).tolist():
        out[c] = out.get(c, 0) + 1
    for c in np.asarray(q_bond).tolist():
        out[c] = out.get(c, 0) - 1
    return {c: v for c, v in out.items() if v > 0}


def _u1_keep(q_sorted, qs, kc):
    """Indices of the first kc[c] directions of every sector c of a charge-sorted leg
    (truncspace(Vk): the target of an oversampled sketch)."""
    idx = []
    for c, k in zip(qs.tolist(), kc.tolist()):
        idx += [i for i, q in enumerate(np.asarray(q_sorted).tolist()) if q == c][:k]
    return np.asarray(idx, dtype=np.int64)


def _sketched_expand_u1(pos, right, psi, H, envs, alg):
    """U(1) SketchedExpand: the steps of `sketched_expand`, each factorisation per charge
    block (oracle.u1), the Gaussian sketch restricted to the charge blocks of the sketched
    complement, and the enlarged bond sorted by charge."""
    from .u1 import fuse, left_orth_u1, right_orth_u1, svd_trunc_u1
    qp = psi.qp
    if right:
        left, rt = psi.ac(pos), psi.AR[pos + 1]
        Dl, d, D = left.shape
        d2, Dn = rt.shape[1], rt.shape[2]
        ql, qr, qn = psi.qb[pos], psi.qb[pos + 1], psi.qb[pos + 2]
        qrow, qcolR = fuse(ql, qp), _col_charges(qp, qn)
        qs, lc, kc = alg.sketch_u1(_u1_comp(qrow, qr), _u1_comp(qcolR, qr))
        l, k = int(lc.sum()), int(kc.sum())
        if k == 0:
            return
        qo = np.repeat(qs, lc)
        lmat = left.reshape(Dl * d, D, order="F")
        RT = rt.reshape(D, d2 * Dn, order="F")
        AL, _, _ = left_orth_u1(lmat, qrow, qr)
        Om = alg.gaussian(Dl * d, l, left.dtype) * (qrow[:, None] == qo[None, :])
        Om, _, _ = left_orth_u1(Om, qrow, qo)
        Q, _, qq = left_orth_u1(Om - AL @ (AL.conj().T @ Om), qrow, qo)
        GLq = dv.transfer_left(envs.leftenv(pos, psi), H[pos], left,
                               Q.reshape(Dl, d, l, order="F"))
        Y = dv.mpo_ac_apply(GLq, H[pos + 1], envs.rightenv(pos + 1, psi), rt)
        B = Y.reshape(l, d2 * Dn, order="F")
        B = B - (B @ RT.conj().T) @ RT
        if l == k:
            _, ar, qa = right_orth_u1(B, qq, qcolR)
        else:
            _, _, Vh, qa, _ = svd_trunc_u1(B, qq, qcolR)
            keep = _u1_keep(qa, qs, kc)
            ar, qa = Vh[keep], qa[keep]
        q = np.concatenate([qr, qa])
        perm = np.argsort(q, kind="stable")
        pad = np.concatenate([lmat, np.zeros((Dl * d, len(qa)), dtype=lmat.dtype)], axis=1)
        nal, nc, qk = left_orth_u1(pad[:, perm], qrow, q[perm])
        assert np.array_equal(qk, q[perm])
        psi.AL[pos] = nal.reshape(Dl, d, len(q), order="F")
        psi.C[pos + 1] = nc / np.linalg.norm(nc)
        psi.AR[pos + 1] = np.concatenate([RT, ar], axis=0)[perm].reshape(len(q), d2, Dn,
                                                                          order="F")
        psi.qb[pos + 1] = q[perm].astype(np.int32)
        psi.center = pos + 1
    else:
        lf, rgt = psi.AL[pos - 1], psi.ac(pos)
        Dp, d, Dl = lf.shape
        d2, Dr = rgt.shape[1], rgt.shape[2]
        qpp, ql, qr = psi.qb[pos - 1], psi.qb[pos], psi.qb[pos + 1]
        qrowL, qcol = fuse(qpp, qp), _col_charges(qp, qr)
        qs, lc, kc = alg.sketch_u1(_u1_comp(qcol, ql), _u1_comp(qrowL, ql))
        l, k = int(lc.sum()), int(kc.sum())
        if k == 0:
            return
        qo = np.repeat(qs, lc)
        lmat = lf.reshape(Dp * d, Dl, order="F")
        RT = rgt.reshape(Dl, d2 * Dr, order="F")
        _, ARtt, _ = right_orth_u1(RT, ql, qcol)
        Om = alg.gaussian(d2 * Dr, l, rgt.dtype) * (qcol[:, None] == qo[None, :])
        Om, _, _ = left_orth_u1(Om, qcol, qo)
        Om = Om.conj().T
        _, Qr, qq = right_orth_u1(Om - (Om @ ARtt.conj().T) @ ARtt, qo, qcol)
        GRq = dv.transfer_right(envs.rightenv(pos, psi), H[pos], rgt,
                                Qr.reshape(l, d2, Dr, order="F"))
        Y = dv.mpo_ac_apply(envs.leftenv(pos - 1, psi), H[pos - 1], GRq, lf)
        B = Y.reshape(Dp * d, l, order="F")
        B = B - lmat @ (lmat.conj().T @ B)
        if l == k:
            Qn, _, qa = left_orth_u1(B, qrowL, qq)
        else:
            U, _, _, qa, _ = svd_trunc_u1(B, qrowL, qq)
            keep = _u1_keep(qa, qs, kc)
            Qn, qa = U[:, keep], qa[keep]
        q = np.concatenate([ql, qa])
        perm = np.argsort(q, kind="stable")
        pad = np.concatenate([RT, np.zeros((len(qa), d2 * Dr), dtype=RT.dtype)], axis=0)
        nc, Qr2, qk = right_orth_u1(pad[perm], q[perm], qcol)
        assert np.array_equal(qk, q[perm])
        psi.AR[pos] = Qr2.reshape(len(q), d2, Dr, order="F")
        psi.C[pos] = nc / np.linalg.norm(nc)
        psi.AL[pos - 1] = np.concatenate([lmat, Qn], axis=1)[:, perm].reshape(Dp, d, len(q),
                                                                              order="F")
        psi.qb[pos] = q[perm].astype(np.int32)
        psi.center = pos


def sketched_expand(pos, right, psi, H, envs, alg):
    """changebond!(site, dir, psi, H, ::SketchedExpand, envs) (sketchedexpand.jl:75-162): a
    random sketch Q of the left (right) complement folded into the left (right) environment
    (transfer with bra Q), one MPO_AC application of the neighbouring site, its projection
    onto that site's complement orthonormalised (LQ / QR, or an SVD truncated back to the
    target when oversampled) and appended to the bond with zero weight."""
    if psi.qb is not None:
        return _sketched_expand_u1(pos, right, psi, H, envs, alg)
    if right:
        left, rt = psi.ac(pos), psi.AR[pos + 1]
        Dl, d, D = left.shape
        d2, Dn = rt.shape[1], rt.shape[2]
        lmat = left.reshape(Dl * d, D, order="F")
        RT = rt.reshape(D, d2 * Dn, order="F")
        AL, _ = qr_pos(lmat)
        compL, compR = Dl * d - D, d2 * Dn - D
        if compL <= 0 or compR <= 0:
            return
        l, k = alg.sketch(compL, compR)
        Om, _ = qr_pos(alg.gaussian(Dl * d, l, left.dtype))          # randisometry
        Q, _ = qr_pos(Om - AL @ (AL.conj().T @ Om))
        GLq = dv.transfer_left(envs.leftenv(pos, psi), H[pos], left,
                               Q.reshape(Dl, d, l, order="F"))         # bra Q, ket AC
        Y = dv.mpo_ac_apply(GLq, H[pos + 1], envs.rightenv(pos + 1, psi), rt)
        B = Y.reshape(l, d2 * Dn, order="F")
        B = B - (B @ RT.conj().T) @ RT
        if l == k:
            _, ar = lq_pos(B)
        else:
            _, _, Vh = np.linalg.svd(B, full_matrices=False)
            ar = Vh[:k]
        kk = ar.shape[0]
        nal, nc = qr_pos(np.concatenate([lmat, np.zeros((Dl * d, kk), dtype=lmat.dtype)], axis=1))
        psi.AL[pos] = nal.reshape(Dl, d, nal.shape[1], order="F")
        psi.C[pos + 1] = nc / np.linalg.norm(nc)
        psi.AR[pos + 1] = np.concatenate([RT, ar], axis=0).reshape(D + kk, d2, Dn, order="F")
        psi.center = pos + 1
    else:
        lf, rgt = psi.AL[pos - 1], psi.ac(pos)
        Dp, d, Dl = lf.shape
        d2, Dr = rgt.shape[1], rgt.shape[2]
        lmat = lf.reshape(Dp * d, Dl, order="F")
        RT = rgt.reshape(Dl, d2 * Dr, order="F")
        _, ARtt = lq_pos(RT)
        compL, compR = Dp * d - Dl, d2 * Dr - Dl
        if compL <= 0 or compR <= 0:
            return
        l, k = alg.sketch(compR, compL)
        Om, _ = qr_pos(alg.gaussian(d2 * Dr, l, rgt.dtype))
        Om = Om.conj().T                                                # adjoint(randisometry)
        _, Qr = lq_pos(Om - (Om @ ARtt.conj().T) @ ARtt)
        GRq = dv.transfer_right(envs.rightenv(pos, psi), H[pos], rgt,
                                Qr.reshape(l, d2, Dr, order="F"))     # bra Qr, ket AC
        Y = dv.mpo_ac_apply(envs.leftenv(pos - 1, psi), H[pos - 1], GRq, lf)
        B = Y.reshape(Dp * d, l, order="F")
        B = B - lmat @ (lmat.conj().T @ B)
        if l == k:
            Qn, _ = qr_pos(B)
        else:
            U, _, _ = np.linalg.svd(B, full_matrices=False)
            Qn = U[:, :k]
        kk = Qn.shape[1]
        nc, Qr2 = lq_pos(np.concatenate([RT, np.zeros((kk, d2 * Dr), dtype=RT.dtype)], axis=0))
        psi.AR[pos] = Qr2.reshape(Qr2.shape[0], d2, Dr, order="F")
        psi.C[pos] = nc / np.linalg.norm(nc)
        psi.AL[pos - 1] = np.concatenate([lmat, Qn], axis=1).reshape(Dp, d, Dl + kk, order="F")
        psi.center = pos


def changebonds(psi, H, alg, envs=None):
    """changebonds!(psi, H, ::OptimalExpand / ::SketchedExpand, envs)
    (optimalexpand.jl:191-199, sketchedexpand.jl:165-173): changebond!(i, :right) at every
    bond from the left (the centre walks right; a positive QR step where nothing is added)."""
    envs = envs or FiniteEnvironments(psi, H)
    expand = sketched_expand if isinstance(alg, SketchedExpand) else optimal_expand
    assert psi.center == 0 or all(a is not None for a in psi.AR)
    psi.center = 0
    for i in range(len(psi) - 1):
        expand(i, True, psi, H, envs, alg)
        if psi.center == i:
            ac = psi.ac(i)
            Dl, d, Dr = ac.shape
            if psi.qb is not None:
                from .u1 import fuse, left_orth_u1
                Q, R, _ = left_orth_u1(ac.reshape(Dl * d, Dr, order="F"),
                                       fuse(psi.qb[i], psi.qp), psi.qb[i + 1])
            else:
                Q, R = qr_pos(ac.reshape(Dl * d, Dr, order="F"))
            psi.AL[i], psi.C[i + 1] = Q.reshape(Dl, d, Q.shape[1], order="F"), R
            psi.center = i + 1
    return psi, envs


class DMRG3S:
    """DMRG3S(noise, ExponentialDecay(decay_rate)) with the truncated SVD DMRG fills in
    (post_expand/dmrg3s.jl:83-153; trunc = truncrank(maxdim) & trunctol(atol)): the noise
    at outer iteration `it` is noise * decay_rate^it (ExponentialDecay, dmrg3s.jl:36-56)."""

    def __init__(self, noise, decay_rate, maxdim, atol=0.0):
        self.noise, self.decay_rate = noise, decay_rate
        self.maxdim, self.atol = maxdim, atol

    def noise_at(self, it):
        return self.noise * self.decay_rate ** it


def dmrg3s_gauge(pos, right, psi, H, envs, AC, noise, maxdim, atol):
    """gauge!(psi, pos, dir, H, envs, AC, ::DMRG3S) (dmrg3s.jl:155-221).  Right: the
    perturbation noise * GL[pos] W[pos] AC with the right bond and the MPO leg fused
    (r fastest) is appended to AC along its right bond, the truncated SVD gives AL[pos] and
    C = S Vh, and AR[pos+1] gets zero rows for the new directions.  Left: the mirror image,
    with the perturbation GR[pos]-side and zero columns appended to AL[pos-1].  For a U(1)
    state the fused leg carries q_bond + q_channel (oracle.u1.mpo_channel_charges), the
    enlarged bond is sorted by charge and the SVD runs block by block.  Returns the
    truncation error."""
    W = H[pos]
    Dl, d, Dr = AC.shape
    if right:
        wr = W.shape[3]
        comb = np.zeros((Dr, wr, Dr * wr), dtype=AC.dtype)   # GR-like: [in, w, out]
        for w in range(wr):
            comb[np.arange(Dr), w, w * Dr + np.arange(Dr)] = 1
        pert = noise * dv.mpo_ac_apply(envs.leftenv(pos, psi), W, comb, AC)
        ACe = np.concatenate([AC, pert], axis=2)
        perm = np.arange(ACe.shape[2])
        if psi.qb is not None:
            # the fused (r, w) leg carries q_r + q_w; the enlarged bond is kept sorted
            from .u1 import fuse, mpo_channel_charges, svd_trunc_u1
            qw = mpo_channel_charges([H[i] for i in range(len(psi))], psi.qp)[pos + 1]
            qe = np.concatenate([psi.qb[pos + 1], fuse(psi.qb[pos + 1], qw)])
            perm = np.argsort(qe, kind="stable")
            U, S, Vh, qk, eps = svd_trunc_u1(ACe[:, :, perm].reshape(Dl * d, -1, order="F"),
                                             fuse(psi.qb[pos], psi.qp), qe[perm], maxdim, atol)
            psi.qb[pos + 1] = qk
        else:
            U, S, Vh, eps = svd_trunc(ACe.reshape(Dl * d, -1, order="F"), maxdim, atol)
        k = S.size
        C = S[:, None] * Vh
        C = C / np.linalg.norm(C)
        B = psi.AR[pos + 1]
        psi.AL[pos] = np.ascontiguousarray(U.reshape(Dl, d, k, order="F"))
        psi.AR[pos + 1] = np.concatenate(
            [B, np.zeros((Dr * wr,) + B.shape[1:], dtype=B.dtype)], axis=0)[perm]
        psi.C[pos + 1] = C
        psi.center = pos + 1
    else:
        wl = W.shape[0]
        comb = np.zeros((Dl * wl, wl, Dl), dtype=AC.dtype)   # GL-like: [out, w, in]
        for w in range(wl):
            comb[w * Dl + np.arange(Dl), w, np.arange(Dl)] = 1
        pert = noise * dv.mpo_ac_apply(comb, W, envs.rightenv(pos, psi), AC)
        ACe = np.concatenate([AC, pert], axis=0)
        perm = np.arange(ACe.shape[0])
        if psi.qb is not None:
            # the fused (l, w) leg carries q_l + q_w
            from .u1 import fuse, mpo_channel_charges, svd_trunc_u1
            qw = mpo_channel_charges([H[i] for i in range(len(psi))], psi.qp)[pos]
            qe = np.concatenate([psi.qb[pos], fuse(psi.qb[pos], qw)])
            perm = np.argsort(qe, kind="stable")
            U, S, Vh, qk, eps = svd_trunc_u1(ACe[perm].reshape(len(qe), d * Dr, order="F"),
                                             qe[perm], _col_charges(psi.qp, psi.qb[pos + 1]),
                                             maxdim, atol)
            psi.qb[pos] = qk
        else:
            U, S, Vh, eps = svd_trunc(ACe.reshape(ACe.shape[0], d * Dr, order="F"), maxdim, atol)
        k = S.size
        C = U * S[None, :]
        C = C / np.linalg.norm(C)
        B = psi.AL[pos - 1]
        psi.AR[pos] = np.ascontiguousarray(Vh.reshape(k, d, Dr, order="F"))
        psi.AL[pos - 1] = np.concatenate(
            [B, np.zeros(B.shape[:2] + (Dl * wl,), dtype=B.dtype)], axis=2)[:, :, perm]
        psi.C[pos] = C
        psi.center = pos
    return eps


def _as_mat(x, nl):
    """Column-major matricisation: first `nl` legs are rows."""
    s = x.shape
    return x.reshape(int(np.prod(s[:nl])), -1, order="F")


def project_complement(Y, AL):
    """Y <- (1 - AL AL') Y on the first two legs (utility.jl:22)."""
    Dl, d, Dm = AL.shape
    Ym = _as_mat(Y, 2)
    A = AL.reshape(Dl * d, Dm, order="F")
    Ym = Ym - A @ (A.conj().T @ Ym)
    return Ym.reshape(Y.shape, order="F")


def dmrg2_local_update(pos, right, psi, H, alg, envs, eps_global, eps_trunc, decay_rate, stats):
    """local_update!(..., ::DMRG2) (dmrg.jl:211-244)."""
    Heff = AC2_hamiltonian(pos, psi, H, envs)
    if right:   # kind = :ACAR
        ac2 = np.einsum("asm,mtb->asbt", psi.ac(pos), psi.AR[pos + 1])
    else:       # kind = :ALAC
        ac2 = np.einsum("asm,mtb->asbt", psi.AL[pos], psi.ac(pos + 1))
    y = Heff(ac2)
    stats["matvecs"] += 1
    y = y / np.linalg.norm(y)
    y = project_complement(y, psi.al(pos))
    eps_local = float(np.linalg.norm(y))
    kd, mi, tol = alg.alg_eigsolve.adapt(decay_rate, eps_local, eps_global, eps_trunc)
    val, new, info = lanczos_eigsolve(Heff, ac2, krylovdim=kd, maxiter=mi, tol=tol,
                                      eager=alg.alg_eigsolve.eager)
    stats["matvecs"] += info.numops
    # gauge2! with truncated SVD (orthoview.jl:401-420)
    Dl, d1, Dr, d2 = new.shape
    M = new.reshape(Dl * d1, Dr * d2, order="F")
    if psi.qb is not None:
        from .u1 import fuse, svd_trunc_u1
        # columns (r, s2): q = q_r - q_s2
        qcol = (np.asarray(psi.qb[pos + 2])[:, None] - np.asarray(psi.qp)[None, :]).reshape(
            -1, order="F")
        U, S, Vh, qk, eps_tr = svd_trunc_u1(M, fuse(psi.qb[pos], psi.qp), qcol, alg.maxdim,
                                            alg.cutoff)
        psi.qb[pos + 1] = qk
    else:
        U, S, Vh, eps_tr = svd_trunc(M, alg.maxdim, alg.cutoff)
    S = S / np.linalg.norm(S)
    k = S.size
    al = U.reshape(Dl, d1, k, order="F")
    ar = np.transpose(Vh.reshape(k, Dr, d2, order="F"), (0, 2, 1))
    C = np.diag(S).astype(psi.dtype)
    psi.AL[pos] = np.ascontiguousarray(al.astype(psi.dtype))
    psi.AR[pos + 1] = np.ascontiguousarray(ar.astype(psi.dtype))
    psi.C[pos + 1] = C
    psi.center = pos + 1
    decay = min(max((info.normres / eps_local) ** (1 / max(1, info.numops)), 1e-3), 0.999) \
        if eps_local > 0 else 0.999
    return eps_local, eps_tr, decay, val


def find_groundstate_dmrg2(psi, H, alg, envs=None, maxsweeps=None, verbose=False):
    """_find_groundstate_sweep! for DMRG2 (dmrg.jl:286-354).  Returns (psi, envs, eps, hist)."""
    psi = psi.copy()
    envs = envs or FiniteEnvironments(psi, H)
    L = len(psi)
    n = L - 1
    eps_locals = np.ones(n)
    eps_global = float(eps_locals.max())
    eps_truncs = np.zeros(n)
    decays = np.zeros(n)
    fwd = list(range(0, L - 1))
    bwd = list(range(L - 3, -1, -1))
    hist = []
    stats = {"matvecs": 0}
    niter = alg.maxiter if maxsweeps is None else maxsweeps
    for it in range(niter):
        for pos in fwd:
            eps_locals[pos], eps_truncs[pos], decays[pos], val = dmrg2_local_update(
                pos, True, psi, H, alg, envs, eps_global, eps_truncs[pos], decays[pos], stats)
            eps_global = float(eps_locals.max())
        for pos in bwd:
            eps_locals[pos], eps_truncs[pos], decays[pos], val = dmrg2_local_update(
                pos, False, psi, H, alg, envs, eps_global, eps_truncs[pos], decays[pos], stats)
            eps_global = float(eps_locals.max())
        eps_global = float(eps_locals.max())
        E = expectation_value_center(psi, H, envs, 0)
        hist.append((it, E, eps_global))
        if verbose:
            print(f"DMRG2 sweep {it}: E={E:.14f} eps={eps_global:.3e}")
        if eps_global <= max(alg.tol, float(eps_truncs.max())):
            break
    return psi, envs, eps_global, hist


def expectation_value_center(psi, H, envs, pos):
    """Energy with the centre at bond pos+1 after a backward sweep (AC[pos] = AL C)."""
    AC = psi.ac(pos)
    Heff = dv.JordanAC(envs.leftenv(pos, psi), H[pos], envs.rightenv(pos, psi))
    return float(np.vdot(AC, Heff(AC)).real / np.vdot(AC, AC).real)


def dmrg1_local_update(pos, right, psi, H, alg, envs, eps_global, eps_trunc, decay_rate, stats):
    """local_update!(..., ::DMRG) with the QR gauge (dmrg.jl:121-158)."""
    ac = psi.ac(pos)
    # calc_galerkin (toolbox.jl:63-70): AC_projection, normalise, project_complement
    Heff = AC_hamiltonian(pos, psi, H, envs)
    y = Heff(ac)
    stats["matvecs"] += 1
    y = y / np.linalg.norm(y)
    # the galerkin error uses the AL of the current centre site
    eps_local = float(np.linalg.norm(project_complement(y, psi.al(pos))))
    if getattr(alg, "alg_expand", None) is not None:
        # 1. expand (dmrg.jl:128-134), then the update from the expanded tensor
        expand = sketched_expand if isinstance(alg.alg_expand, SketchedExpand) else optimal_expand
        expand(pos, right, psi, H, envs, alg.alg_expand)
        ac = psi.ac(pos)
        Heff = AC_hamiltonian(pos, psi, H, envs)
    Dl, d, Dr = ac.shape
    kd, mi, tol = alg.alg_eigsolve.adapt(decay_rate, eps_local, eps_global, eps_trunc)
    val, new, info = lanczos_eigsolve(Heff, ac, krylovdim=kd, maxiter=mi, tol=tol,
                                      eager=alg.alg_eigsolve.eager)
    stats["matvecs"] += info.numops
    g = getattr(alg, "alg_gauge", None)
    if g is not None:
        noise = g.noise_at(stats.get("iter", 0))
        if noise != 0.0:
            eps_tr = dmrg3s_gauge(pos, right, psi, H, envs, new, noise, g.maxdim, g.atol)
            decay = min(max((info.normres / eps_local) ** (1 / max(1, info.numops)), 1e-3),
                        0.999) if eps_local > 0 else 0.999
            return eps_local, eps_tr, decay, val
    if right:
        if psi.qb is not None:
            from .u1 import fuse, left_orth_u1
            Q, R, qk = left_orth_u1(new.reshape(Dl * d, Dr, order="F"), fuse(psi.qb[pos], psi.qp),
                                    psi.qb[pos + 1])
            assert np.array_equal(qk, psi.qb[pos + 1]), "QR changed a bond space"
        else:
            Q, R = qr_pos(new.reshape(Dl * d, Dr, order="F"))
        R = R / np.linalg.norm(R)
        psi.AL[pos] = Q.reshape(Dl, d, Dr, order="F")
        psi.C[pos + 1] = R
        psi.center = pos + 1
    else:
        if psi.qb is not None:
            from .u1 import right_orth_u1
            Lm, Q, qk = right_orth_u1(new.reshape(Dl, d * Dr, order="F"), psi.qb[pos],
                                      _col_charges(psi.qp, psi.qb[pos + 1]))
            assert np.array_equal(qk, psi.qb[pos]), "LQ changed a bond space"
        else:
            Lm, Q = lq_pos(new.reshape(Dl, d * Dr, order="F"))
        Lm = Lm / np.linalg.norm(Lm)
        psi.AR[pos] = Q.reshape(Dl, d, Dr, order="F")
        psi.C[pos] = Lm
        psi.center = pos
    decay = min(max((info.normres / eps_local) ** (1 / max(1, info.numops)), 1e-3), 0.999) \
        if eps_local > 0 else 0.999
    return eps_local, 0.0, decay, val


def find_groundstate_dmrg(psi, H, alg, envs=None, maxsweeps=None):
    """_find_groundstate_sweep! for single-site DMRG (dmrg.jl:250-354)."""
    psi = psi.copy()
    envs = envs or FiniteEnvironments(psi, H)
    L = len(psi)
    eps_locals = np.ones(L)
    eps_global = 1.0
    decays = np.zeros(L)
    stats = {"matvecs": 0}
    hist = []
    niter = alg.maxiter if maxsweeps is None else maxsweeps
    for it in range(niter):
        stats["iter"] = it
        for pos in range(0, L - 1):
            eps_locals[pos], _, decays[pos], val = dmrg1_local_update(
                pos, True, psi, H, alg, envs, eps_global, 0.0, decays[pos], stats)
            eps_global = float(eps_locals.max())
        for pos in range(L - 1, 0, -1):
            eps_locals[pos], _, decays[pos], val = dmrg1_local_update(
                pos, False, psi, H, alg, envs, eps_global, 0.0, decays[pos], stats)
            eps_global = float(eps_locals.max())
        E = float(val)
        hist.append((it, E, eps_global))
        if eps_global <= alg.tol:
            break
    return psi, envs, eps_global, hist


# ---------------------------------------------------------------- TDVP (finite, 1-site)

def tdvp_timestep(psi, H, envs, t, dt, krylovdim=30, tol=1e-10, imaginary=False):
    """_timestep_finite! (tdvp.jl:147-211): left-to-right half-step sweep with backward bond
    evolutions, the right edge, the mirrored right-to-left sweep and the left edge.
    integrate(H, y, t, dt) = exp(-i dt H) y (exp(-dt H) in imaginary time), integrators.jl:44-53."""
    from .krylov import lanczos_exponentiate

    def integ(op, y, d):
        tt = -d if imaginary else -1j * d
        out, _ = lanczos_exponentiate(op, tt, y, krylovdim=krylovdim, tol=tol)
        return out

    L = len(psi)
    psi.ac_site = None
    for i in range(L - 1):
        AC = integ(AC_hamiltonian(i, psi, H, envs), psi.ac(i), dt / 2)
        Dl, d, Dr = AC.shape
        Q, R = qr_pos(AC.reshape(Dl * d, Dr, order="F"))
        psi.AL[i] = Q.reshape(Dl, d, -1, order="F")
        psi.C[i + 1] = R
        psi.center = i + 1
        psi.ac_site = None
        Hc = dv.CHam(envs.leftenv(i + 1, psi), envs.rightenv(i, psi))
        psi.C[i + 1] = integ(Hc, psi.C[i + 1], -dt / 2)
    psi.ac_tensor = integ(AC_hamiltonian(L - 1, psi, H, envs), psi.ac(L - 1), dt / 2)
    psi.ac_site = L - 1
    for i in range(L - 1, 0, -1):
        AC = integ(AC_hamiltonian(i, psi, H, envs), psi.ac(i), dt / 2)
        Dl, d, Dr = AC.shape
        Lm, Q = lq_pos(AC.reshape(Dl, d * Dr, order="F"))
        psi.AR[i] = Q.reshape(-1, d, Dr, order="F")
        psi.C[i] = Lm
        psi.center = i
        psi.ac_site = None
        Hc = dv.CHam(envs.leftenv(i, psi), envs.rightenv(i - 1, psi))
        psi.C[i] = integ(Hc, psi.C[i], -dt / 2)
    psi.ac_tensor = integ(AC_hamiltonian(0, psi, H, envs), psi.ac(0), dt / 2)
    psi.ac_site = 0
    return psi, envs
