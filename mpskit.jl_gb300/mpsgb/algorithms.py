"""Ground-state drivers on the device (host mirror of MPSKit's DMRG / DMRG2).

  DMRG / DMRG2 local_update! and the sweep  -- src/algorithms/groundstate/dmrg.jl:121-354
  AdaptiveKrylov / adapt_solver             -- src/utility/dynamictols.jl:182-235
  calc_galerkin                             -- src/algorithms/toolbox.jl:63-70
  expectation_value(FiniteMPS, H)           -- src/algorithms/expval.jl:136-141
  OptimalExpand changebond!                 -- src/algorithms/changebonds/optimalexpand.jl:122-187
  DMRG3S gauge!, ExponentialDecay           -- src/algorithms/post_expand/dmrg3s.jl:36-56, 133-192
"""
import math
import time

import numpy as np

from . import _lib as L
from .core import DeviceTensor
from .derivatives import (AC2_hamiltonian, AC_hamiltonian, C_hamiltonian, GB300Backend, Lanczos,
                          exponentiate, fixedpoint, mpo_projection, transfer_left,
                          transfer_right)
from .states import (FiniteEnvironments, ac2_from, left_orth, mps_cat, mps_permute, mul_front,
                     mul_tail, perturb, project_complement_, project_complement_right_,
                     right_orth, svd_trunc)

EPS34 = np.finfo(np.float64).eps ** 0.75


class AdaptiveKrylov:
    """Per-bond adaptive Krylov budget (dynamictols.jl:130-235), same defaults."""

    def __init__(self, krylovdim_min=3, krylovdim_max=20, iter_min=1, iter_max=1,
                 tol_min=1e-12, tol_max=1e-2, truncation_factor=1e-1, tol_factor=1e-1,
                 eager=True):
        if not (0 < krylovdim_min <= krylovdim_max):
            raise ValueError("need 0 < krylovdim_min <= krylovdim_max")
        if not (1 <= iter_min <= iter_max):
            raise ValueError("need 1 <= iter_min <= iter_max")
        self.krylovdim_min, self.krylovdim_max = krylovdim_min, krylovdim_max
        self.iter_min, self.iter_max = iter_min, iter_max
        self.tol_min, self.tol_max = tol_min, tol_max
        self.truncation_factor, self.tol_factor = truncation_factor, tol_factor
        self.eager = eager

    def adapt(self, decay_rate=0.0, g_local=0.0, g_global=0.0, eps_trunc=0.0):
        tol = min(max(max(self.truncation_factor * eps_trunc, self.tol_factor * g_global),
                      self.tol_min), self.tol_max)
        rho = min(max(decay_rate, 0.0), 1.0)
        if not (0.0 < rho < 1.0):
            if rho == 0.0:
                return Lanczos(self.krylovdim_min, self.iter_min, tol, self.eager)
            return Lanczos(self.krylovdim_max, self.iter_max, tol, self.eager)
        R = max(g_local, self.tol_min) / tol
        nmat = int(round(math.log(R) / math.log(1.0 / rho)))
        kd = min(max(nmat, self.krylovdim_min), self.krylovdim_max)
        mi = min(max(-((-5 * nmat) // (2 * kd)) - 3, self.iter_min), self.iter_max)
        return Lanczos(kd, mi, tol, self.eager)


class DMRG2:
    def __init__(self, maxdim, cutoff=0.0, tol=1e-10, maxiter=200, alg_eigsolve=None,
                 backend=None, verbosity=0):
        self.maxdim, self.cutoff = maxdim, cutoff
        self.tol, self.maxiter = tol, maxiter
        self.alg_eigsolve = alg_eigsolve or AdaptiveKrylov()
        self.backend = backend or GB300Backend()
        self.verbosity = verbosity


class DMRG:
    """Single-site DMRG (dmrg.jl:55-158).  alg_gauge = None: the positive QR/LQ gauge;
    a DMRG3S: the perturbed, truncated gauge.  alg_expand = an OptimalExpand run ahead of
    every local update (dmrg.jl:128-134)."""

    def __init__(self, tol=1e-10, maxiter=200, alg_eigsolve=None, backend=None, verbosity=0,
                 alg_gauge=None, alg_expand=None):
        self.tol, self.maxiter = tol, maxiter
        self.alg_eigsolve = alg_eigsolve or AdaptiveKrylov()
        self.backend = backend or GB300Backend()
        self.verbosity = verbosity
        self.alg_gauge = alg_gauge
        self.alg_expand = alg_expand


class OptimalExpand:
    """OptimalExpand(; trunc = truncrank(add)) (optimalexpand.jl:36-47): at most `add`
    directions are added to a bond per expansion."""

    def __init__(self, add):
        self.add = add


class DMRG3S:
    """DMRG3S(noise, ExponentialDecay(decay_rate)) with the truncated SVD DMRG fills in
    (dmrg3s.jl:83-131; trunc = truncrank(maxdim) & trunctol(atol)): the noise at outer
    iteration `it` is noise * decay_rate^it."""

    def __init__(self, noise, decay_rate, maxdim, atol=0.0):
        self.noise, self.decay_rate = noise, decay_rate
        self.maxdim, self.atol = maxdim, atol

    def noise_at(self, it):
        return self.noise * self.decay_rate ** it


def optimal_expand(pos, right, psi, H, envs, alg, backend=None):
    """changebond!(site, dir, psi, H, ::OptimalExpand, envs) (optimalexpand.jl:122-187):
    the two-site update AC2_projection projected onto the complements of both sites, its
    `add` dominant right (left) singular directions appended to the bond with zero weight
    -- the state is unchanged -- and the site regauged.  The complements are applied as
    projectors (1 - AL AL') Y (1 - AR' AR) instead of null-space bases: the singular
    vectors of the projected Y are those of NL' Y NR' mapped back by NL / NR.  Directions
    whose singular value is below eps^(3/4) of the normalised Y (arbitrary in the
    reference) are not added.  For a U(1) state the SVD runs per charge block and the
    enlarged bond is re-sorted by charge (gb_mps_permute), as TensorKit's catdomain /
    catcodomain keeps a graded space sorted."""
    backend = backend or GB300Backend()
    b = pos if right else pos - 1
    if right:
        left, rt = psi.ac(pos), psi.AR[pos + 1]
        PL = psi.al(pos)
    else:
        left, rt = psi.AL[pos - 1], psi.ac(pos)
        PL = left
    # two-site update from the projected effective Hamiltonian (AC2_projection)
    Y = AC2_hamiltonian(b, psi, H, envs, backend)(ac2_from(left, rt))
    project_complement_(Y, PL)
    if right:
        project_complement_right_(Y, rt)
    else:
        # the right complement of AC[pos]: its row space is that of its LQ factor
        _, q = right_orth(rt)
        project_complement_right_(Y, q)
    nrm = Y.norm()
    if nrm <= EPS34:
        return
    Y.scale_(1.0 / nrm)
    u, _, vh, _ = svd_trunc(Y, alg.add, EPS34, normalize=False)
    u1 = rt.charges is not None and left.charges is not None
    if right:
        k = vh.dims[0]
        nar = mps_cat(rt, vh, 0)                         # AR[pos+1] with the new rows
        pad = mps_cat(left, None, 2, nb=k)               # [AC | 0]
        if u1:
            q = np.concatenate([rt.charges[0], vh.charges[0]])
            perm = np.argsort(q, kind="stable")
            nar = mps_permute(nar, 0, perm, (q[perm], rt.charges[1], rt.charges[2]))
            pad = mps_permute(pad, 2, perm, (left.charges[0], left.charges[1], q[perm]))
        nal, nc = left_orth(pad)                         # regauged
        nc.scale_(1.0 / nc.norm())
        psi.AL[pos], psi.C[pos + 1], psi.AR[pos + 1] = nal, nc, nar
        psi.center = pos + 1
    else:
        k = u.dims[2]
        nal = mps_cat(left, u, 2)                        # AL[pos-1] with the new columns
        pad = mps_cat(rt, None, 0, nb=k)                 # [AC ; 0]
        if u1:
            q = np.concatenate([left.charges[2], u.charges[2]])
            perm = np.argsort(q, kind="stable")
            nal = mps_permute(nal, 2, perm, (left.charges[0], left.charges[1], q[perm]))
            pad = mps_permute(pad, 0, perm, (q[perm], rt.charges[1], rt.charges[2]))
        nc, nar = right_orth(pad)                        # regauged
        nc.scale_(1.0 / nc.norm())
        psi.AL[pos - 1], psi.C[pos], psi.AR[pos] = nal, nc, nar
        psi.center = pos


class SketchedExpand:
    """SketchedExpand(; trunc = truncrank(add), oversampling) (sketchedexpand.jl:41-73):
    `add` directions per bond from a random sketch of `add + oversampling` columns.  The
    random isometries are drawn on the host from numpy's PCG64 seeded with `seed`, one
    Gaussian matrix per expansion in call order, and orthonormalised on the device."""

    def __init__(self, add, oversampling=0, seed=0):
        self.add, self.oversampling = add, oversampling
        self.rng = np.random.default_rng(seed)

    def gaussian(self, m, n, dtype):
        g = self.rng.standard_normal((m, n))
        if np.dtype(dtype).kind == "c":
            g = g + 1j * self.rng.standard_normal((m, n))
        return g.astype(dtype)

    def sketch(self, comp, other):
        """(l, k): sketch columns and target directions in the sketched complement `comp`,
        both capped by the other site's complement (beyond it the new directions could not
        stay orthogonal to the state)."""
        cap = min(comp, other)
        k = min(self.add, cap)
        return min(k + self.oversampling, cap), k

    def sketch_u1(self, comp, other):
        """The U(1) form of `sketch`: `comp`, `other` map charge -> complement dimension.
        sample_space (randexpand.jl:160-165) gives every direction of the (capped) complement
        a uniform random weight and keeps the `add` largest -- a uniform random subset, whose
        per-sector counts are k_c; the oversampling adds up to `oversampling` directions in
        every sector (sketch_space, sketchedexpand.jl:61-66).  Returns (charges, l_c, k_c)."""
        qs = [c for c in sorted(comp) if min(comp[c], other.get(c, 0)) > 0]
        cap = np.array([min(comp[c], other[c]) for c in qs], dtype=np.int64)
        tot = int(cap.sum())
        w = self.rng.random(tot)
        keep = np.argsort(-w, kind="stable")[:min(self.add, tot)]
        kc = np.bincount(np.repeat(np.arange(len(qs)), cap)[keep], minlength=len(qs))
        return np.asarray(qs, dtype=np.int32), np.minimum(cap, kc + self.oversampling), kc


def _complement_dims(q_fused, q_bond):
    """charge -> dimension of the complement of a bond inside a fused leg (U(1))."""
    u, n = np.unique(np.asarray(q_fused), return_counts=True)
    out = dict(zip(u.tolist(), n.tolist()))
    for c, m in zip(*np.unique(np.asarray(q_bond), return_counts=True)):
        out[int(c)] = out.get(int(c), 0) - int(m)
    return {c: v for c, v in out.items() if v > 0}


def _fuse(qa, qb):
    return (np.asarray(qa)[:, None] + np.asarray(qb)[None, :]).reshape(-1, order="F").astype(
        np.int32)


def _sector_select(q_sorted, qs, kc, dtype, ctx):
    """The 0/1 bond matrix (k x n) picking, in every charge sector of a charge-sorted leg
    whose directions come in descending singular value, its first kc[c] directions
    (truncspace(Vk) of the reference).  Returns (matrix, charges of the kept directions)."""
    q_sorted = np.asarray(q_sorted)
    idx = []
    for c, k in zip(qs.tolist(), kc.tolist()):
        idx += np.nonzero(q_sorted == c)[0][:k].tolist()
    S = np.zeros((len(idx), len(q_sorted)), dtype=dtype)
    S[np.arange(len(idx)), idx] = 1
    return DeviceTensor.from_numpy(ctx, L.GB_KIND_BOND, S), q_sorted[idx].astype(np.int32)


def sketched_expand(pos, right, psi, H, envs, alg, backend=None):
    """changebond!(site, dir, psi, H, ::SketchedExpand, envs) (sketchedexpand.jl:75-162):
    a random sketch Q of one site's complement folded into that site's environment (a
    transfer with bra Q), one MPO_AC projection of the neighbouring site (gb_mpo_project),
    projected onto the neighbour's complement and orthonormalised (LQ / QR, or a truncated
    SVD when oversampled), then appended to the bond with zero weight: the state is
    unchanged.  At single-site cost: no two-site tensor is formed.  For a U(1) state the
    sketch is drawn per charge sector (`SketchedExpand.sketch_u1`), every factorisation runs
    per block, an oversampled sketch is cut back to k_c directions in each sector, and the
    enlarged bond is re-sorted by charge (gb_mps_permute)."""
    backend = backend or GB300Backend()
    ctx = envs.ctx
    W = H.device(ctx, envs.dtype)
    if right:
        left, rt = psi.ac(pos), psi.AR[pos + 1]
        Dl, d, D = left.dims
        d2, Dn = rt.dims[1], rt.dims[2]
        u1 = left.charges is not None and rt.charges is not None
        if u1:
            ql, qp, qr = left.charges
            qn, qp2 = rt.charges[2], rt.charges[1]
            qrow = _fuse(ql, qp)
            qs, lc, kc = alg.sketch_u1(_complement_dims(qrow, qr),
                                       _complement_dims(_fuse(-np.asarray(qp2), qn), qr))
            l, k = int(lc.sum()), int(kc.sum())
            if k == 0:
                return
            qo = np.repeat(qs, lc).astype(np.int32)
            g = alg.gaussian(Dl * d, l, left.dtype) * (qrow[:, None] == qo[None, :])
            G = DeviceTensor.from_numpy(ctx, L.GB_KIND_MPS, g.reshape(Dl, d, l, order="F"))
            G.charges = (ql, qp, qo)
        else:
            compL, compR = Dl * d - D, d2 * Dn - D
            if compL <= 0 or compR <= 0:
                return
            l, k = alg.sketch(compL, compR)
            G = DeviceTensor.from_numpy(ctx, L.GB_KIND_MPS, alg.gaussian(Dl * d, l, left.dtype)
                                        .reshape(Dl, d, l, order="F"))
        AL = psi.al(pos)
        Om, _ = left_orth(G)                                   # randisometry
        Q, _ = left_orth(project_complement_(Om, AL))          # qr_compact of the complement part
        GLq = transfer_left(envs.leftenv(pos, psi), W[pos], left, Q, backend)
        Y = mpo_projection(GLq, envs.rightenv(pos + 1, psi), rt, W[pos + 1], backend=backend)
        if u1:
            Y.charges = (Q.charges[2], qp2, qn)
        project_complement_right_(Y, rt)
        if l == k:
            _, ar = right_orth(Y)
        else:
            Y.reshape_(L.GB_KIND_AC2, (l, 1, Dn, d2))
            if u1:
                Y.charges = (Q.charges[2], np.zeros(1, np.int32), qn, qp2)
                _, _, arf, _ = svd_trunc(Y, None, 0.0, normalize=False)
                Sel, qsel = _sector_select(arf.charges[0], qs, kc, arf.dtype, ctx)
                ar = mul_front(Sel, arf)
                ar.charges = (qsel, qp2, qn)
            else:
                _, _, ar, _ = svd_trunc(Y, k, 0.0, normalize=False)
        kk = ar.dims[0]
        nar = mps_cat(rt, ar, 0)
        pad = mps_cat(left, None, 2, nb=kk)
        if u1:
            q = np.concatenate([qr, ar.charges[0]])
            perm = np.argsort(q, kind="stable")
            nar = mps_permute(nar, 0, perm, (q[perm], qp2, qn))
            pad = mps_permute(pad, 2, perm, (ql, qp, q[perm]))
        nal, nc = left_orth(pad)
        nc.scale_(1.0 / nc.norm())
        psi.AL[pos], psi.C[pos + 1], psi.AR[pos + 1] = nal, nc, nar
        psi.center = pos + 1
    else:
        lf, rgt = psi.AL[pos - 1], psi.ac(pos)
        Dp, d, Dl = lf.dims
        d2, Dr = rgt.dims[1], rgt.dims[2]
        u1 = lf.charges is not None and rgt.charges is not None
        if u1:
            qpp, qp = lf.charges[0], lf.charges[1]
            ql, qp2, qr = rgt.charges
            qcol = _fuse(-np.asarray(qp2), qr)
            qs, lc, kc = alg.sketch_u1(_complement_dims(qcol, ql),
                                       _complement_dims(_fuse(qpp, qp), ql))
            l, k = int(lc.sum()), int(kc.sum())
            if k == 0:
                return
            qo = np.repeat(qs, lc).astype(np.int32)
            g = alg.gaussian(d2 * Dr, l, rgt.dtype) * (qcol[:, None] == qo[None, :])
        else:
            compL, compR = Dp * d - Dl, d2 * Dr - Dl
            if compL <= 0 or compR <= 0:
                return
            l, k = alg.sketch(compR, compL)
            g = alg.gaussian(d2 * Dr, l, rgt.dtype)
        _, ARtt = right_orth(rgt)
        G = DeviceTensor.from_numpy(ctx, L.GB_KIND_MPS, g.reshape(1, d2 * Dr, l, order="F"))
        if u1:
            G.charges = (np.zeros(1, np.int32), qcol, qo)
        Om, _ = left_orth(G)                                   # randisometry (d2 Dr) x l
        from .infinite import adjoint
        Om = adjoint(Om.reshape_(L.GB_KIND_BOND, (d2 * Dr, l)))
        Om.reshape_(L.GB_KIND_MPS, (l, d2, Dr))                # its adjoint, l x (s r)
        if u1:
            Om.charges = (qo, qp2, qr)
        _, Qr = right_orth(project_complement_right_(Om, ARtt))
        GRq = transfer_right(envs.rightenv(pos, psi), W[pos], rgt, Qr, backend)
        Y = mpo_projection(envs.leftenv(pos - 1, psi), GRq, lf, W[pos - 1], backend=backend)
        if u1:
            Y.charges = (qpp, qp, Qr.charges[0])
        project_complement_(Y, lf)
        if l == k:
            Qn, _ = left_orth(Y)
        else:
            Y.reshape_(L.GB_KIND_AC2, (Dp, d, l, 1))
            if u1:
                Y.charges = (qpp, qp, Qr.charges[0], np.zeros(1, np.int32))
                Qf, _, _, _ = svd_trunc(Y, None, 0.0, normalize=False)
                Sel, qsel = _sector_select(Qf.charges[2], qs, kc, Qf.dtype, ctx)
                Qn = mul_tail(Qf, adjoint(Sel))
                Qn.charges = (qpp, qp, qsel)
            else:
                Qn, _, _, _ = svd_trunc(Y, k, 0.0, normalize=False)
        kk = Qn.dims[2]
        nal = mps_cat(lf, Qn, 2)
        pad = mps_cat(rgt, None, 0, nb=kk)
        if u1:
            q = np.concatenate([ql, Qn.charges[2]])
            perm = np.argsort(q, kind="stable")
            nal = mps_permute(nal, 2, perm, (qpp, qp, q[perm]))
            pad = mps_permute(pad, 0, perm, (q[perm], qp2, qr))
        nc, nar = right_orth(pad)
        nc.scale_(1.0 / nc.norm())
        psi.AL[pos - 1], psi.C[pos], psi.AR[pos] = nal, nc, nar
        psi.center = pos


def changebonds(psi, H, alg, envs=None, backend=None):
    """changebonds!(psi, H, ::OptimalExpand / ::SketchedExpand, envs)
    (optimalexpand.jl:191-199, sketchedexpand.jl:165-173): changebond!(i, :right) at every
    bond from the left.  The state is changed in place (only its gauge and bond spaces: the
    added directions carry zero weight); the centre bond walks from the left end to the right
    end, with a positive QR step where a bond has nothing to add.  Returns (psi, envs)."""
    envs = envs or FiniteEnvironments(psi, H)
    expand = sketched_expand if isinstance(alg, SketchedExpand) else optimal_expand
    psi.right_canonicalize(0)
    for i in range(len(psi) - 1):
        expand(i, True, psi, H, envs, alg, backend)
        if psi.center == i:
            q, R = left_orth(psi.ac(i))
            psi.AL[i], psi.C[i + 1], psi.center = q, R, i + 1
    return psi, envs


def dmrg3s_gauge(pos, right, psi, H, envs, AC, noise, maxdim, atol):
    """gauge!(psi, pos, dir, H, envs, AC, ::DMRG3S) (dmrg3s.jl:133-192).  Right: the
    perturbation noise * GL[pos] W[pos] AC with the right bond and the MPO channel fused
    (bond index fastest) is appended to AC along its right bond, the truncated SVD gives
    AL[pos] and C = S Vh, and AR[pos+1] gets zero rows for the new directions.  Left: the
    mirror image with GR[pos], zero columns appended to AL[pos-1].  For a U(1) state the fused
    leg carries q_bond + q_channel (the channel charges of the MPO), the enlarged bond is
    re-sorted by charge (gb_mps_permute) and the SVD runs per charge block.  Returns the
    truncation error."""
    W = H.device(envs.ctx, envs.dtype)[pos]
    Dl, d, Dr = AC.dims
    u1 = AC.charges is not None
    if u1:
        ql, qp, qr = (np.asarray(q, np.int32) for q in AC.charges)
        qw = H.channel_charges(qp)
    if right:
        P = perturb(envs.leftenv(pos, psi), W, AC, 0, envs.precision)
        P.scale_(noise)
        ACe = mps_cat(AC, P, 2)
        De = ACe.dims[2]
        if u1:
            qe = np.concatenate([qr, (qr[:, None] + qw[pos + 1][None, :]).reshape(-1, order="F")])
            perm = np.argsort(qe, kind="stable")
            qe = qe[perm].astype(np.int32)
            ACe = mps_permute(ACe, 2, perm)
        ACe.reshape_(L.GB_KIND_AC2, (Dl, d, De, 1))             # left_gauge as an SVD
        if u1:
            ACe.charges = (ql, qp, qe, np.zeros(1, np.int32))
        al, S, vh, eps = svd_trunc(ACe, maxdim, atol, normalize=True)
        k = S.dims[0]
        C = mul_front(S, vh)
        C.reshape_(L.GB_KIND_BOND, (k, De))
        ar = mps_cat(psi.AR[pos + 1], None, 0, nb=P.dims[2])
        if u1:
            C.charges = (S.charges[0], qe)
            qa = psi.AR[pos + 1].charges
            ar = mps_permute(ar, 0, perm, (qe, qa[1], qa[2]))
        psi.AL[pos] = al
        psi.AR[pos + 1] = ar
        psi.C[pos + 1] = C
        psi.center = pos + 1
    else:
        P = perturb(envs.rightenv(pos, psi), W, AC, 1, envs.precision)
        P.scale_(noise)
        ACe = mps_cat(AC, P, 0)
        De = ACe.dims[0]
        if u1:
            qe = np.concatenate([ql, (ql[:, None] + qw[pos][None, :]).reshape(-1, order="F")])
            perm = np.argsort(qe, kind="stable")
            qe = qe[perm].astype(np.int32)
            ACe = mps_permute(ACe, 0, perm)
        ACe.reshape_(L.GB_KIND_AC2, (De, 1, Dr, d))             # right_gauge as an SVD
        if u1:
            ACe.charges = (qe, np.zeros(1, np.int32), qr, qp)
        u, S, ar, eps = svd_trunc(ACe, maxdim, atol, normalize=True)
        k = S.dims[0]
        C = mul_tail(u, S)
        C.reshape_(L.GB_KIND_BOND, (De, k))
        al = mps_cat(psi.AL[pos - 1], None, 2, nb=P.dims[0])
        if u1:
            C.charges = (qe, S.charges[1])
            qa = psi.AL[pos - 1].charges
            al = mps_permute(al, 2, perm, (qa[0], qa[1], qe))
        psi.AR[pos] = ar
        psi.AL[pos - 1] = al
        psi.C[pos] = C
        psi.center = pos
    return eps


def _decay(normres, eps_local, numops):
    if eps_local <= 0:
        return 0.999
    return min(max((normres / eps_local) ** (1.0 / max(1, numops)), 1e-3), 0.999)


class SweepStats:
    """Counters of a sweep; with sync=True the phase timers synchronise the device so
    the per-phase times are exact (at the cost of host/device overlap)."""

    def __init__(self, sync=False):
        self.sync = sync
        self.matvecs = 0
        self.updates = 0
        self.heff_flops = 0.0
        self.t = {"heff_build": 0.0, "eigsolve": 0.0, "gauge": 0.0, "env": 0.0}


def dmrg2_local_update(pos, right, psi, H, alg, envs, eps_global, eps_trunc, decay_rate, stats):
    """local_update!(..., ::DMRG2) (dmrg.jl:211-244)."""
    def now():
        if stats.sync:
            psi.ctx.synchronize()
        return time.perf_counter()

    t0 = now()
    Heff = AC2_hamiltonian(pos, psi, H, envs, alg.backend)
    t1 = now()
    ac2 = ac2_from(psi.ac(pos), psi.AR[pos + 1]) if right else ac2_from(psi.AL[pos], psi.ac(pos + 1))
    y = Heff(ac2)
    y.normalize_()
    project_complement_(y, psi.al(pos))
    eps_local = y.norm()
    solver = alg.alg_eigsolve.adapt(decay_rate, eps_local, eps_global, eps_trunc)
    val, new, info = fixedpoint(Heff, ac2, "SR", solver)
    t2 = now()
    al, S, ar, eps_tr = svd_trunc(new, alg.maxdim, alg.cutoff, normalize=True)
    psi.AL[pos] = al
    psi.AR[pos + 1] = ar
    psi.C[pos + 1] = S
    psi.center = pos + 1
    t3 = now()
    stats.matvecs += info.numops + 1
    stats.updates += 1
    stats.heff_flops += Heff.flops * (info.numops + 1)
    stats.t["heff_build"] += t1 - t0
    stats.t["eigsolve"] += t2 - t1
    stats.t["gauge"] += t3 - t2
    return eps_local, eps_tr, _decay(info.normres, eps_local, info.numops), val


def expectation_value(psi, H, envs, site=0, backend=None):
    """<psi|H|psi>/<psi|psi> contracted at a site adjacent to the centre."""
    ac = psi.ac(site)
    Heff = AC_hamiltonian(site, psi, H, envs, backend or GB300Backend())
    return float(np.real(ac.dot(Heff(ac)) / ac.dot(ac)))


def variance(psi, H, envs=None, backend=None):
    """variance(state::FiniteMPS, H) (toolbox.jl:125-128): <H H> - <H>^2, with H H the
    MPO product (its own environments)."""
    envs = envs or FiniteEnvironments(psi, H)
    site = min(psi.center, len(psi) - 1)
    e = expectation_value(psi, H, envs, site, backend)
    H2 = H * H
    e2 = expectation_value(psi, H2, FiniteEnvironments(psi, H2), site, backend)
    return float(e2 - e * e)


def find_groundstate(psi, H, alg, envs=None, maxsweeps=None, callback=None):
    """find_groundstate(psi, H, DMRG2()/DMRG()/GradientGrassmann()) on the device.  DMRG
    modifies the input state in place (find_groundstate! semantics); GradientGrassmann
    returns a new state (gradient_grassmann.jl:80-121).  Returns (psi, envs, eps, history):
    eps is the truncation error of DMRG, the final gradient norm of GradientGrassmann."""
    from .grassmann import GradientGrassmann, find_groundstate_grassmann
    if isinstance(alg, GradientGrassmann):
        return find_groundstate_grassmann(psi, H, alg, envs)
    if isinstance(alg, DMRG2):
        return _sweep_dmrg2(psi, H, alg, envs, maxsweeps, callback)
    if isinstance(alg, DMRG):
        return _sweep_dmrg1(psi, H, alg, envs, maxsweeps, callback)
    raise TypeError("unsupported algorithm")


def _sweep_dmrg2(psi, H, alg, envs, maxsweeps, callback):
    envs = envs or FiniteEnvironments(psi, H)
    envs.precision = alg.backend.code
    n = len(psi) - 1
    eps_locals = np.ones(n)
    eps_truncs = np.zeros(n)
    decays = np.zeros(n)
    eps_global = float(eps_locals.max())
    fwd = list(range(0, len(psi) - 1))
    bwd = list(range(len(psi) - 3, -1, -1))
    hist = []
    stats = SweepStats()
    niter = alg.maxiter if maxsweeps is None else maxsweeps
    for it in range(niter):
        t0 = time.perf_counter()
        for right, rng in ((True, fwd), (False, bwd)):
            for pos in rng:
                eps_locals[pos], eps_truncs[pos], decays[pos], _ = dmrg2_local_update(
                    pos, right, psi, H, alg, envs, eps_global, eps_truncs[pos], decays[pos], stats)
                eps_global = float(eps_locals.max())
        E = expectation_value(psi, H, envs, 0, alg.backend)
        dt = time.perf_counter() - t0
        hist.append({"sweep": it, "energy": float(np.real(E)), "eps": eps_global, "time": dt,
                     "matvecs": stats.matvecs})
        if alg.verbosity:
            print(f"DMRG2 sweep {it}: E = {np.real(E):.14f}  eps = {eps_global:.3e}  t = {dt:.3f}s")
        if callback:
            callback(it, psi, envs)
        if eps_global <= max(alg.tol, float(eps_truncs.max())):
            break
    return psi, envs, eps_global, hist


def dmrg1_local_update(pos, right, psi, H, alg, envs, eps_global, decay_rate, it):
    """local_update!(..., ::DMRG) (dmrg.jl:121-158): Galerkin error, optional expansion,
    eigensolve, then the QR/LQ or the DMRG3S gauge."""
    ac = psi.ac(pos)
    Heff = AC_hamiltonian(pos, psi, H, envs, alg.backend)
    y = Heff(ac)
    y.normalize_()
    project_complement_(y, psi.al(pos))
    eps_local = y.norm()
    if alg.alg_expand is not None:
        expand = sketched_expand if isinstance(alg.alg_expand, SketchedExpand) else optimal_expand
        expand(pos, right, psi, H, envs, alg.alg_expand, alg.backend)
        ac = psi.ac(pos)
        Heff = AC_hamiltonian(pos, psi, H, envs, alg.backend)
    solver = alg.alg_eigsolve.adapt(decay_rate, eps_local, eps_global, 0.0)
    val, new, info = fixedpoint(Heff, ac, "SR", solver)
    decay = _decay(info.normres, eps_local, info.numops)
    g = alg.alg_gauge
    if g is not None and g.noise_at(it) != 0.0:
        eps_tr = dmrg3s_gauge(pos, right, psi, H, envs, new, g.noise_at(it), g.maxdim, g.atol)
        return eps_local, eps_tr, decay, val
    if right:
        q, R = left_orth(new)
        R.scale_(1.0 / R.norm())
        psi.AL[pos] = q
        psi.C[pos + 1] = R
        psi.center = pos + 1
    else:
        Lm, q = right_orth(new)
        Lm.scale_(1.0 / Lm.norm())
        psi.AR[pos] = q
        psi.C[pos] = Lm
        psi.center = pos
    return eps_local, 0.0, decay, val


def _sweep_dmrg1(psi, H, alg, envs, maxsweeps, callback):
    envs = envs or FiniteEnvironments(psi, H)
    envs.precision = alg.backend.code
    n = len(psi)
    eps_locals = np.ones(n)
    decays = np.zeros(n)
    eps_global = 1.0
    hist = []
    niter = alg.maxiter if maxsweeps is None else maxsweeps
    val = 0.0
    for it in range(niter):
        for right, rng in ((True, range(0, n - 1)), (False, range(n - 1, 0, -1))):
            for pos in rng:
                eps_locals[pos], _, decays[pos], val = dmrg1_local_update(
                    pos, right, psi, H, alg, envs, eps_global, decays[pos], it)
                eps_global = float(eps_locals.max())
        hist.append({"sweep": it, "energy": float(val), "eps": eps_global})
        if callback:
            callback(it, psi, envs)
        if eps_global <= alg.tol:
            break
    return psi, envs, eps_global, hist


# ---------------------------------------------------------------- TDVP

class TDVP:
    """Single-site TDVP (src/algorithms/timestep/tdvp.jl:30-60) with the KrylovKit
    Lanczos exponentiator of Defaults.alg_expsolve (krylovdim 30, tol 1e-10)."""

    def __init__(self, integrator=None, backend=None):
        self.integrator = integrator or Lanczos(krylovdim=30, maxiter=200, tol=1e-10)
        self.backend = backend or GB300Backend()


def timestep(psi, H, t, dt, alg, envs=None, imaginary_evolution=False):
    """timestep!(psi::FiniteMPS, H, t, dt, TDVP()) (tdvp.jl:135-211) on the device:
    forward half-step sweep with backward bond evolutions, the right edge, the mirrored
    backward sweep and the left edge.  Returns (psi, envs)."""
    envs = envs or FiniteEnvironments(psi, H)
    envs.precision = alg.backend.code
    n = len(psi)

    def integ(op, y, d):
        tt = -d if imaginary_evolution else -1j * d
        out, info = exponentiate(op, tt, y, alg.integrator)
        return out

    psi.ac_site = None
    for i in range(n - 1):
        AC = integ(AC_hamiltonian(i, psi, H, envs, alg.backend), psi.ac(i), dt / 2)
        q, R = left_orth(AC)
        psi.AL[i] = q
        psi.C[i + 1] = R
        psi.center = i + 1
        psi.ac_site = None
        Hc = C_hamiltonian(i, psi, H, envs, alg.backend)
        psi.C[i + 1] = integ(Hc, psi.C[i + 1], -dt / 2)
    psi.ac_tensor = integ(AC_hamiltonian(n - 1, psi, H, envs, alg.backend), psi.ac(n - 1), dt / 2)
    psi.ac_site = n - 1
    for i in range(n - 1, 0, -1):
        AC = integ(AC_hamiltonian(i, psi, H, envs, alg.backend), psi.ac(i), dt / 2)
        Lm, q = right_orth(AC)
        psi.AR[i] = q
        psi.C[i] = Lm
        psi.center = i
        psi.ac_site = None
        Hc = C_hamiltonian(i - 1, psi, H, envs, alg.backend)
        psi.C[i] = integ(Hc, psi.C[i], -dt / 2)
    psi.ac_tensor = integ(AC_hamiltonian(0, psi, H, envs, alg.backend), psi.ac(0), dt / 2)
    psi.ac_site = 0
    return psi, envs
