"""U(1)-symmetric factorisations on dense-embedded tensors (oracle; test infrastructure).

A U(1)-symmetric TensorMap is stored as one dense array with charge-sorted legs and exact
zeros outside the charge-conserving blocks (MPS tensor A[l s; r]: q_l + q_s = q_r).
TensorKit (not vendored in the reference; compat 0.17.1) factorises a symmetric TensorMap
block by block -- MatrixAlgebraKit's `left_orth`, `right_orth` and `svd_trunc` act on each
coupled-charge block of `blocks(t)` -- and a truncation strategy ranks the singular values
of all blocks together.  Call sites in the reference: left_gauge / right_gauge
(src/states/orthoview.jl:322-339), gauge2! with svd_trunc (src/states/orthoview.jl:401-420),
the FiniteMPS QR sweep (src/states/finitemps.jl:234-237).

Ties among singular values at the truncation edge are broken by charge, then by position
in the block, as in the library.
"""
import numpy as np

from .mps import lq_pos, qr_pos


def fuse(qa, qb):
    """q[a + Da*b] = qa[a] + qb[b] (column-major fused leg)."""
    return (np.asarray(qa)[:, None] + np.asarray(qb)[None, :]).reshape(-1, order="F")


def sectors(qrow, qcol):
    """[(charge, row indices, col indices)] for charges present on both sides, ascending."""
    qrow, qcol = np.asarray(qrow), np.asarray(qcol)
    out = []
    for c in sorted(set(qrow.tolist()) & set(qcol.tolist())):
        out.append((c, np.nonzero(qrow == c)[0], np.nonzero(qcol == c)[0]))
    return out


def _check_blocks(M, secs):
    inside = sum(np.linalg.norm(M[np.ix_(r, c)]) ** 2 for _, r, c in secs)
    full = np.linalg.norm(M) ** 2
    assert full - inside <= 1e-10 * full + 1e-300, "weight outside the charge blocks"


def left_orth_u1(M, qrow, qcol):
    """M = Q R per block (positive QR).  Returns Q (m x k), R (k x n), new bond charges."""
    secs = sectors(qrow, qcol)
    _check_blocks(M, secs)
    k = sum(min(len(r), len(c)) for _, r, c in secs)
    Q = np.zeros((M.shape[0], k), dtype=M.dtype)
    R = np.zeros((k, M.shape[1]), dtype=M.dtype)
    qk = np.zeros(k, dtype=np.int32)
    o = 0
    for q, r, c in secs:
        Qc, Rc = qr_pos(M[np.ix_(r, c)])
        kc = Qc.shape[1]
        Q[np.ix_(r, np.arange(o, o + kc))] = Qc
        R[np.ix_(np.arange(o, o + kc), c)] = Rc
        qk[o:o + kc] = q
        o += kc
    return Q, R, qk


def right_orth_u1(M, qrow, qcol):
    """M = L Q per block (positive LQ).  Returns L (m x k), Q (k x n), new bond charges."""
    secs = sectors(qrow, qcol)
    _check_blocks(M, secs)
    k = sum(min(len(r), len(c)) for _, r, c in secs)
    Lm = np.zeros((M.shape[0], k), dtype=M.dtype)
    Q = np.zeros((k, M.shape[1]), dtype=M.dtype)
    qk = np.zeros(k, dtype=np.int32)
    o = 0
    for q, r, c in secs:
        Lc, Qc = lq_pos(M[np.ix_(r, c)])
        kc = Qc.shape[0]
        Lm[np.ix_(r, np.arange(o, o + kc))] = Lc
        Q[np.ix_(np.arange(o, o + kc), c)] = Qc
        qk[o:o + kc] = q
        o += kc
    return Lm, Q, qk


def svd_trunc_u1(M, qrow, qcol, maxdim=None, atol=0.0):
    """Blockwise SVD with truncrank(maxdim) & trunctol(atol) over all blocks.
    Returns U (m x k), S (k), Vh (k x n), new bond charges, eps (norm of the discarded)."""
    secs = sectors(qrow, qcol)
    _check_blocks(M, secs)
    facs = []
    ranked = []
    for ci, (q, r, c) in enumerate(secs):
        U, S, Vh = np.linalg.svd(M[np.ix_(r, c)], full_matrices=False)
        facs.append((U, S, Vh))
        ranked += [(-s, ci, j) for j, s in enumerate(S)]
    ranked.sort()
    sv = np.array([-t[0] for t in ranked])
    keep = int(np.sum(sv > atol))
    if maxdim is not None:
        keep = min(keep, maxdim)
    keep = max(keep, 1)
    eps = float(np.linalg.norm(sv[keep:]))
    kc = [0] * len(secs)
    for _, ci, _j in ranked[:keep]:
        kc[ci] += 1
    U = np.zeros((M.shape[0], keep), dtype=M.dtype)
    Vh = np.zeros((keep, M.shape[1]), dtype=M.dtype)
    S = np.zeros(keep)
    qk = np.zeros(keep, dtype=np.int32)
    o = 0
    for ci, (q, r, c) in enumerate(secs):
        n = kc[ci]
        if n == 0:
            continue
        Uc, Sc, Vc = facs[ci]
        cols = np.arange(o, o + n)
        U[np.ix_(r, cols)] = Uc[:, :n]
        Vh[np.ix_(cols, c)] = Vc[:n]
        S[o:o + n] = Sc[:n]
        qk[o:o + n] = q
        o += n
    return U, S, Vh, qk, eps


def mpo_channel_charges(W, qp):
    """Channel charges of a finite MPO with charge-definite channels (TensorKit's graded MPO
    spaces; the DMRG3S combiner fuses a bond with them, post_expand/dmrg3s.jl:122-131).
    W[a, s, t, c] != 0 (s bra, t ket) fixes q_c = q_a + q_s - q_t.  Forward sweep from the
    charge-0 left boundary, then a backward sweep from the charge-0 right boundary for channels
    reached only from the right; unlinked channels carry 0."""
    qp = [int(x) for x in qp]
    q = [dict() for _ in range(len(W) + 1)]
    q[0] = {a: 0 for a in range(W[0].shape[0])}
    q[-1] = {c: 0 for c in range(W[-1].shape[3])}
    nzs = [np.argwhere(np.asarray(w) != 0) for w in W]
    for i, nz in enumerate(nzs):                       # forward
        for a, s, t, c in nz:
            if a in q[i]:
                v = q[i][a] + qp[s] - qp[t]
                assert q[i + 1].setdefault(c, v) == v, "channel without a definite charge"
    for i in range(len(W) - 1, -1, -1):                # backward
        for a, s, t, c in nzs[i]:
            if c in q[i + 1]:
                v = q[i + 1][c] - qp[s] + qp[t]
                assert q[i].setdefault(a, v) == v, "channel without a definite charge"
    dims = [W[0].shape[0]] + [w.shape[3] for w in W]
    return [np.array([q[b].get(c, 0) for c in range(dims[b])], dtype=np.int32)
            for b in range(len(W) + 1)]
