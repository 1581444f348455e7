"""Effective local operators (derivative operators) -- oracle restatement.

Restates src/algorithms/derivatives/hamiltonian_derivatives.jl (Jordan-form AC / AC2),
src/algorithms/derivatives/mpo_derivatives.jl (generic C / AC / AC2 and their
prepared forms) and src/transfermatrix/transfer.jl:125-130 (MPO transfer).

Every @plansor of the reference is written as an np.einsum with the same index
pattern.  For the dense (Trivial-symmetry) spaces used here, planar contraction
equals ordinary contraction and conj() is the elementwise conjugate.

Leg orders: GL[a, w, a'], GR[b', w, b], W[wl, s, s', wr], x_AC[l, s, r],
x_AC2[l, s1, r, s2], x_C[l, r].
"""
import numpy as np

TERMS_AC2 = ("II", "IC", "ID", "CB", "CA", "AB", "AA", "BE", "DE", "EE")
TERMS_AC = ("D", "I", "E", "C", "B", "A")


def _nz(x):
    return x is not None and x.size > 0 and bool(np.any(x != 0))


def jordan_blocks(W):
    """A, B, C, D blocks of a Jordan MPO tensor (jordanmpotensor.jl:44-249).

    A = W[2:end-1, 1, 1, 2:end-1], B = W[2:end-1, ..., end], C = W[1, ..., 2:end-1],
    D = W[1, ..., end] (1-based).  With one row (one column) only, the single row is
    the start row (the single column is the finished column).
    """
    A = W[1:-1, :, :, 1:-1]
    B = W[1:-1, :, :, -1]          # (c, s, s')
    C = W[0, :, :, 1:-1]           # (s, s', k)
    D = W[0, :, :, -1]             # (s, s')
    return A, B, C, D


def connected_channels(A1, A2):
    """_connected_channels (hamiltonian_derivatives.jl:243-270), at flat channel level.

    Returns (rows, mids, cols) as ascending index arrays or None."""
    if not (_nz(A1) and _nz(A2)):
        return None
    nz1 = np.any(A1 != 0, axis=(1, 2))   # (rows, mids)
    nz2 = np.any(A2 != 0, axis=(1, 2))   # (mids, cols)
    fed = np.any(nz1, axis=0)
    feeds = np.any(nz2, axis=1)
    both = fed & feeds
    mids = np.nonzero(both)[0]
    if mids.size == 0:
        return None
    rows = np.nonzero(np.any(nz1[:, both], axis=1))[0]
    cols = np.nonzero(np.any(nz2[both, :], axis=0))[0]
    return rows, mids, cols


# ------------------------------------------------------------------ generic MPO forms

def mpo_c_apply(GL, GR, x):
    """MPO_C_Hamiltonian apply (mpo_derivatives.jl:92-98):
    y[-1;-2] = GL[-1 3;1] x[1;2] GR[2 3;-2]."""
    return np.einsum("awc,cd,dwb->ab", GL, x, GR, optimize=True)


def mpo_ac_apply(GL, W, GR, x):
    """MPO_AC_Hamiltonian apply (mpo_derivatives.jl:100-107):
    y[-1 -2;-3] = GL[-1 5;4] x[4 2;1] W[5 -2;2 3] GR[1 3;-3],
    evaluated in the prepared order of mpo_derivatives.jl:221-231, 266-274:
    L = GL*W fused to (l s) <- (w' l' s'), then y = L (x R)."""
    # GL_O[a, s, w', a', s'] = GL[a, w, a'] W[w, s, s', w']
    GLO = np.tensordot(GL, W, axes=([1], [0]))          # (a, a', s, s', w')
    GLO = GLO.transpose(0, 2, 4, 1, 3)                   # (a, s, w', a', s')
    # xR[a', s', w', b] = x[a', s', b'] GR[b', w', b]
    xR = np.tensordot(x, GR, axes=([2], [0]))            # (a', s', w', b)
    return np.tensordot(GLO, xR, axes=([2, 3, 4], [2, 0, 1]))   # (a, s, b)


def mpo_ac2_apply(GL, W1, W2, GR, x):
    """MPO_AC2_Hamiltonian apply (mpo_derivatives.jl:144-153):
    y[-1 -2;-3 -4] = GL[-1 7;6] x[6 5;1 3] W1[7 -2;5 4] W2[4 -4;3 2] GR[1 2;-3],
    evaluated as the prepared operator (mpo_derivatives.jl:233-247, 276-288):
    GL_O[l s1 m; l' s1'] = GL[l c; l'] W1[c s1; s1' m],
    O_GR[r' s2'; r s2 m] = W2[m s2; s2' c'] GR[r' c'; r],
    y = GL_O . x . O_GR as two GEMMs."""
    GLO = np.tensordot(GL, W1, axes=([1], [0]))          # (l, l', s1, s1', m)
    GLO = GLO.transpose(0, 2, 4, 1, 3)                   # (l, s1, m, l', s1')
    OGR = np.tensordot(W2, GR, axes=([3], [1]))          # (m, s2, s2', r', r)
    OGR = OGR.transpose(3, 2, 4, 1, 0)                   # (r', s2', r, s2, m)
    # T[l, s1, m, r', s2'] = GL_O[(l s1 m), (l' s1')] x[(l' s1'), (r' s2')]
    T = np.tensordot(GLO, x, axes=([3, 4], [0, 1]))      # (l, s1, m, r', s2')
    # y[l, s1, r, s2] = T[(l s1), (m r' s2')] O_GR[(m r' s2'), (r s2)]
    return np.tensordot(T, OGR, axes=([2, 3, 4], [4, 0, 1]))    # (l, s1, r, s2)


# ------------------------------------------------------------------ Jordan AC2

class JordanAC2:
    """JordanMPO_AC2_Hamiltonian (hamiltonian_derivatives.jl:168-217, 272-369) with
    `prepare_operator!!` (:371-468) and the matvec (:485-500)."""

    def __init__(self, GL, W1, W2, GR, prepare=True):
        A1, B1, C1, D1 = jordan_blocks(W1)
        A2, B2, C2, D2 = jordan_blocks(W2)
        GL2 = GL[:, 1:-1, :]
        GR2 = GR[:, 1:-1, :]
        cplx = np.iscomplexobj(GL) or np.iscomplexobj(GR) or np.iscomplexobj(W1)
        self.dtype = np.complex128 if cplx else np.float64
        t = {}
        # not started (:284): transpose(removeunit(GR[1], 2)) -> II[r, r'] = GR[r', 0, r]
        t["II"] = None if W2.shape[3] == 1 else GR[:, 0, :].T.copy()
        # finished (:287)
        t["EE"] = None if W1.shape[0] == 1 else GL[:, -1, :].copy()
        # starting right (:290-295): IC[-1 -2;-3 -4] = C2[-1;-3 1] GR2[-4 1;-2]
        t["IC"] = np.einsum("suk,vkb->sbuv", C2, GR2, optimize=True) if _nz(C2) else None
        t["DE"] = D1.copy() if _nz(D1) else None
        t["ID"] = D2.copy() if _nz(D2) else None
        # CB[-1 -2;-3 -4] = C1[-1;-3 1] B2[1 -2;-4]  (:304-310)
        t["CB"] = np.einsum("suk,ktv->stuv", C1, B2, optimize=True) if (_nz(C1) and _nz(B2)) else None
        # CA[-1 -2 -3;-4 -5 -6] = C1[-1;-4 1] A2[1 -2;-5 2] GR2[-6 2;-3]  (:313-319)
        t["CA"] = (np.einsum("suk,ktgm,qmr->strugq", C1, A2, GR2, optimize=True)
                   if (_nz(C1) and _nz(A2)) else None)
        # AB[-1 -2 -3;-4 -5 -6] = GL2[-1 2;-4] A1[2 -2;-5 1] B2[1 -3;-6]  (:322-328)
        t["AB"] = (np.einsum("acl,csuk,ktv->astluv", GL2, A1, B2, optimize=True)
                   if (_nz(A1) and _nz(B2)) else None)
        # BE[-1 -2;-3 -4] = GL2[-1 2;-3] B1[2 -2;-4]  (:331-336)
        t["BE"] = np.einsum("acl,csu->aslu", GL2, B1, optimize=True) if _nz(B1) else None
        ch = connected_channels(A1, A2)
        if ch is None:
            t["AA"] = None
        else:
            rows, mids, cols = ch
            t["AA"] = (GL2[:, rows, :], A1[np.ix_(rows, range(A1.shape[1]), range(A1.shape[2]), mids)],
                       A2[np.ix_(mids, range(A2.shape[1]), range(A2.shape[2]), cols)], GR2[:, cols, :])
        for k in ("IC", "CB", "CA", "AB", "BE", "II", "EE", "DE", "ID"):
            if t[k] is not None:
                t[k] = t[k].astype(self.dtype)
        self.t = t
        if prepare:
            self._prepare()

    def _prepare(self):
        """prepare_operator!! (hamiltonian_derivatives.jl:371-468): fold the cheap terms
        into the 3,3 (CA/AB) or 2,2 (IC/BE) terms."""
        t = self.t
        CA, AB = t["CA"], t["AB"]
        # CB (:379-389)
        if CA is not None and t["CB"] is not None:
            D = CA.shape[2]
            CA += np.einsum("stuv,rq->struvq", t["CB"], np.eye(D), optimize=True)
            t["CB"] = None
        elif AB is not None and t["CB"] is not None:
            D = AB.shape[0]
            AB += np.einsum("stuv,al->astluv", t["CB"], np.eye(D), optimize=True)
            t["CB"] = None
        # IC into CA (:392-398)
        if CA is not None and t["IC"] is not None:
            d = CA.shape[0]
            CA += np.einsum("su,tbvq->stbuvq", np.eye(d), t["IC"], optimize=True)
            t["IC"] = None
        # BE into AB (:401-407)
        if AB is not None and t["BE"] is not None:
            d = AB.shape[2]
            AB += np.einsum("aslu,tv->astluv", t["BE"], np.eye(d), optimize=True)
            t["BE"] = None
        # DE (:410-422)
        if t["BE"] is not None and t["DE"] is not None:
            D = t["BE"].shape[0]
            t["BE"] += np.einsum("al,su->aslu", np.eye(D), t["DE"], optimize=True)
            t["DE"] = None
        elif AB is not None and t["DE"] is not None:
            D, d = AB.shape[0], AB.shape[2]
            AB += np.einsum("al,su,tv->astluv", np.eye(D), t["DE"], np.eye(d), optimize=True)
            t["DE"] = None
        # ID (:425-436)
        if t["IC"] is not None and t["ID"] is not None:
            D = t["IC"].shape[1]
            t["IC"] += np.einsum("su,bq->sbuq", t["ID"], np.eye(D), optimize=True)
            t["ID"] = None
        elif CA is not None and t["ID"] is not None:
            d, D = CA.shape[0], CA.shape[2]
            CA += np.einsum("su,tv,rq->struvq", np.eye(d), t["ID"], np.eye(D), optimize=True)
            t["ID"] = None
        # II (:439-449)
        if t["IC"] is not None and t["II"] is not None:
            d = t["IC"].shape[0]
            t["IC"] += np.einsum("su,bq->sbuq", np.eye(d), t["II"], optimize=True)
            t["II"] = None
        elif CA is not None and t["II"] is not None:
            d = CA.shape[0]
            CA += np.einsum("su,tv,rq->struvq", np.eye(d), np.eye(d), t["II"], optimize=True)
            t["II"] = None
        # EE (:452-462)
        if t["BE"] is not None and t["EE"] is not None:
            d = t["BE"].shape[1]
            t["BE"] += np.einsum("al,su->aslu", t["EE"], np.eye(d), optimize=True)
            t["EE"] = None
        elif AB is not None and t["EE"] is not None:
            d = AB.shape[1]
            AB += np.einsum("al,su,tv->astluv", t["EE"], np.eye(d), np.eye(d), optimize=True)
            t["EE"] = None

    def terms(self):
        return tuple(k for k in TERMS_AC2 if self.t[k] is not None)

    def __call__(self, x):
        """Matvec (hamiltonian_derivatives.jl:485-500)."""
        t = self.t
        x = np.asarray(x)
        dt = np.result_type(x.dtype, self.dtype)
        if t["AA"] is not None:
            GL2, A1, A2, GR2 = t["AA"]
            y = mpo_ac2_apply(GL2, A1, A2, GR2, x).astype(dt)
        else:
            y = np.zeros(x.shape, dtype=dt)
        if t["II"] is not None:   # y[-1 -2;-3 -4] += x[-1 -2;1 -4] II[-3;1]
            y += np.einsum("apqr,bq->apbr", x, t["II"], optimize=True)
        if t["IC"] is not None:   # y += x[-1 -2;1 2] IC[-4 -3;2 1]
            y += np.einsum("apqu,rbuq->apbr", x, t["IC"], optimize=True)
        if t["ID"] is not None:   # y += x[-1 -2;-3 1] ID[-4;1]
            y += np.einsum("apbu,ru->apbr", x, t["ID"], optimize=True)
        if t["CB"] is not None:   # y += x[-1 1;-3 2] CB[-2 -4;1 2]
            y += np.einsum("aubv,pruv->apbr", x, t["CB"], optimize=True)
        if t["CA"] is not None:   # y += x[-1 1;3 2] CA[-2 -4 -3;1 2 3]
            y += np.einsum("auqv,prbuvq->apbr", x, t["CA"], optimize=True)
        if t["AB"] is not None:   # y += x[1 2;-3 3] AB[-1 -2 -4;1 2 3]
            y += np.einsum("lubv,aprluv->apbr", x, t["AB"], optimize=True)
        if t["BE"] is not None:   # y += x[1 2;-3 -4] BE[-1 -2;1 2]
            y += np.einsum("lubr,aplu->apbr", x, t["BE"], optimize=True)
        if t["DE"] is not None:   # y += x[-1 1;-3 -4] DE[-2;1]
            y += np.einsum("aubr,pu->apbr", x, t["DE"], optimize=True)
        if t["EE"] is not None:   # y += x[1 -2;-3 -4] EE[-1;1]
            y += np.einsum("lpbr,al->apbr", x, t["EE"], optimize=True)
        return y


# ------------------------------------------------------------------ Jordan AC

class JordanAC:
    """JordanMPO_AC_Hamiltonian (hamiltonian_derivatives.jl:15-107), prepare (:109-157)
    and matvec (:472-483)."""

    def __init__(self, GL, W, GR, prepare=True):
        A, B, C, D = jordan_blocks(W)
        GL2 = GL[:, 1:-1, :]
        GR2 = GR[:, 1:-1, :]
        cplx = np.iscomplexobj(GL) or np.iscomplexobj(GR) or np.iscomplexobj(W)
        self.dtype = np.complex128 if cplx else np.float64
        t = {}
        t["D"] = D.copy() if _nz(D) else None
        # I = removeunit(GR[1], 2) -> I[r', r] (used as x[-1 -2;1] I[1;-3])
        t["I"] = None if W.shape[3] == 1 else GR[:, 0, :].copy()
        t["E"] = None if W.shape[0] == 1 else GL[:, -1, :].copy()
        # starting[-1 -2;-3 -4] = WC[-1;-3 1] GR2[-4 1;-2]  (:77-82)
        t["C"] = np.einsum("suk,vkb->sbuv", C, GR2, optimize=True) if _nz(C) else None
        # ending[-1 -2;-3 -4] = GL2[-1 1;-3] WB[1 -2;-4]  (:85-90)
        t["B"] = np.einsum("acl,csu->aslu", GL2, B, optimize=True) if _nz(B) else None
        t["A"] = (GL2, A, GR2) if _nz(A) else None
        for k in ("D", "I", "E", "C", "B"):
            if t[k] is not None:
                t[k] = t[k].astype(self.dtype)
        self.t = t
        if prepare:
            self._prepare()

    def _prepare(self):
        t = self.t
        if t["D"] is not None:
            if t["C"] is not None:      # C[-1 -2;-3 -4] += D[-1;-3] Id[-2;-4]
                D = t["C"].shape[1]
                t["C"] += np.einsum("su,bq->sbuq", t["D"], np.eye(D), optimize=True)
                t["D"] = None
            elif t["B"] is not None:    # B[-1 -2;-3 -4] += Id[-1;-3] D[-2;-4]
                D = t["B"].shape[0]
                t["B"] += np.einsum("al,su->aslu", np.eye(D), t["D"], optimize=True)
                t["D"] = None
        if t["I"] is not None and t["C"] is not None:   # C += Id[-1;-3] I[-4;-2]
            d = t["C"].shape[0]
            t["C"] += np.einsum("su,qb->sbuq", np.eye(d), t["I"], optimize=True)
            t["I"] = None
        if t["E"] is not None and t["B"] is not None:   # B += E[-1;-3] Id[-2;-4]
            d = t["B"].shape[1]
            t["B"] += np.einsum("al,su->aslu", t["E"], np.eye(d), optimize=True)
            t["E"] = None

    def terms(self):
        return tuple(k for k in TERMS_AC if self.t[k] is not None)

    def __call__(self, x):
        t = self.t
        dt = np.result_type(x.dtype, self.dtype)
        if t["A"] is not None:
            GL2, A, GR2 = t["A"]
            y = mpo_ac_apply(GL2, A, GR2, x).astype(dt)
        else:
            y = np.zeros(x.shape, dtype=dt)
        if t["D"] is not None:  # y[-1 -2;-3] += x[-1 1;-3] D[-2;1]
            y += np.einsum("aub,su->asb", x, t["D"], optimize=True)
        if t["E"] is not None:  # y += E[-1;1] x[1 -2;-3]
            y += np.einsum("al,lsb->asb", t["E"], x, optimize=True)
        if t["I"] is not None:  # y += x[-1 -2;1] I[1;-3]
            y += np.einsum("asq,qb->asb", x, t["I"], optimize=True)
        if t["C"] is not None:  # y += x[-1 2;1] C[-2 -3;2 1]
            y += np.einsum("auq,sbuq->asb", x, t["C"], optimize=True)
        if t["B"] is not None:  # y += B[-1 -2;1 2] x[1 2;-3]
            y += np.einsum("aslu,lub->asb", t["B"], x, optimize=True)
        return y


class CHam:
    """MPO_C_Hamiltonian (mpo_derivatives.jl:20-23, 92-98); prepared form is the same map."""

    def __init__(self, GL, GR):
        self.GL, self.GR = GL, GR

    def __call__(self, x):
        return mpo_c_apply(self.GL, self.GR, x)


# ------------------------------------------------------------------ transfers

def transfer_left(GL, W, A, Ab):
    """transfer_left(x, O, A, Ab) (transfer.jl:125-127):
    y[-1 -2;-3] = x[1 2;4] A[4 5;-3] O[2 3;5 -2] conj(Ab[1 3;-1])."""
    # as three pairwise contractions (a four-operand einsum can fall back to a naive loop)
    T1 = np.tensordot(GL, A, axes=([2], [0]))                # (p, w, t, b)
    T2 = np.tensordot(T1, W, axes=([1, 2], [0, 2]))          # (p, b, s, v)
    return np.tensordot(Ab.conj(), T2, axes=([0, 1], [0, 2])).transpose(0, 2, 1)  # (a, v, b)


def transfer_right(GR, W, A, Ab):
    """transfer_right(v, O, A, Ab) (transfer.jl:128-130):
    v[-1 -2;-3] = A[-1 2;1] O[-2 4;2 3] conj(Ab[-3 4;5]) v[1 3;5]."""
    T1 = np.tensordot(A, GR, axes=([2], [0]))                # (a, t, v, r)
    T2 = np.tensordot(T1, W, axes=([1, 2], [2, 3]))          # (a, r, w, s)
    return np.tensordot(T2, Ab.conj(), axes=([3, 1], [1, 2]))  # (a, w, b)


def contract_mpo_expval(AC, GL, W, GR):
    """contract_mpo_expval (expval.jl:96-100):
    GL[1 2;3] AC[3 7;5] GR[5 8;6] O[2 4;7 8] conj(AC[1 4;6])."""
    return np.einsum("abc,cge,ehf,bdgh,adf->", GL, AC, GR, W, AC.conj(), optimize=True)
