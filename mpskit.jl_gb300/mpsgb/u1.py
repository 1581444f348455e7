"""U(1) symmetry on the dense device tensors.

TensorKit stores a U(1)-symmetric TensorMap (`U1Irrep` sectors) as one dense block per
coupled charge.  Here the same tensor is one dense array whose virtual legs are sorted by
charge, with exact zeros outside the charge-conserving blocks:

    MPS tensor A[l s; r]       q_l + q_s = q_r
    bond tensor C[l; r]        q_l = q_r
    two-site AC2[l s1; r s2]   q_l + q_s1 + q_s2 = q_r

Charge flows left to right: the left boundary carries 0, the right boundary the total
charge Q (2 Sz for spin 1/2).  Every contraction is then an ordinary dense contraction whose
zero tiles the split-precision GEMM skips (its operands' nonzero maps), and the
factorisations (`gb_u1_left_orth`, `gb_u1_right_orth`, `gb_u1_svd_trunc`) act per block so
that the zeros stay exact.  A `DeviceTensor` carries its leg charges in `charges`.
"""
import numpy as np

from .operators import SPIN_HALF_CHARGES


def fuse(qa, qb):
    """Charges of the column-major fused leg (a, b): q[a + Da*b] = qa[a] + qb[b]."""
    qa, qb = np.asarray(qa), np.asarray(qb)
    return (qa[:, None] + qb[None, :]).reshape(-1, order="F")


def block_mask(*legs, signs=None):
    """Boolean mask of the charge-conserving entries of a tensor with the given leg charges:
    sum_i signs[i] q_i = 0 (default signs: +1 for every leg but the last, -1 for the last)."""
    n = len(legs)
    signs = signs or [1] * (n - 1) + [-1]
    tot = np.zeros([len(q) for q in legs], dtype=np.int64)
    for i, (q, s) in enumerate(zip(legs, signs)):
        shape = [1] * n
        shape[i] = len(q)
        tot = tot + s * np.asarray(q, dtype=np.int64).reshape(shape)
    return tot == 0


def bond_charges(L, D, Q=0, qphys=SPIN_HALF_CHARGES):
    """Charge-sorted virtual spaces of an L-site chain with total charge Q: bond b (b sites
    to its left) holds the charges reachable from both ends, each sector no larger than its
    full-rank dimension, sector sizes following a Gaussian profile of variance b(L-b)/L
    (the binomial-like distribution of a random-walk bridge), total at most D."""
    qphys = np.asarray(qphys, dtype=np.int64)
    out = []
    counts_left = {0: 1}
    lefts = [dict(counts_left)]
    for b in range(L):
        nxt = {}
        for q, c in counts_left.items():
            for p in qphys:
                nxt[q + p] = nxt.get(q + p, 0) + c
        counts_left = nxt
        lefts.append(dict(counts_left))
    counts_right = {Q: 1}
    rights = [None] * (L + 1)
    rights[L] = dict(counts_right)
    for b in range(L - 1, -1, -1):
        nxt = {}
        for q, c in counts_right.items():
            for p in qphys:
                nxt[q - p] = nxt.get(q - p, 0) + c
        counts_right = nxt
        rights[b] = dict(counts_right)
    for b in range(L + 1):
        qs = sorted(set(lefts[b]) & set(rights[b]))
        # full-rank sector dimensions (capped at D: the counts grow like 2^b)
        full = np.array([min(lefts[b][q], rights[b][q], D) for q in qs], dtype=np.int64)
        if full.sum() <= D:
            dims = full.copy()
        else:
            var = max(b * (L - b) / L, 0.25)
            mean = Q * b / L
            w = np.exp(-(np.array(qs, dtype=np.float64) - mean) ** 2 / (2 * var))
            dims = np.maximum(1, np.floor(D * w / w.sum())).astype(np.int64)
            dims = np.minimum(dims, full)
            # hand out what is left to the largest sectors that still have room
            order = np.argsort(-w, kind="stable")
            left = D - int(dims.sum())
            while left > 0:
                moved = False
                for i in order:
                    if left == 0:
                        break
                    if dims[i] < full[i]:
                        dims[i] += 1
                        left -= 1
                        moved = True
                if not moved:
                    break
            while dims.sum() > D:  # more sectors than D: drop the lightest ones
                i = int(np.argmin(np.where(dims > 0, w, np.inf)))
                dims[i] -= 1
        out.append(np.repeat(np.array(qs, dtype=np.int32), dims))
    return out


def random_u1_tensors(L, D, seed, Q=0, dtype=np.float64, qphys=SPIN_HALF_CHARGES):
    """Seeded i.i.d. normal entries (PCG64) on the charge-conserving blocks of the spaces of
    `bond_charges`; returns (tensors, bond charges)."""
    rng = np.random.default_rng(seed)
    qb = bond_charges(L, D, Q, qphys)
    As = []
    for i in range(L):
        shape = (len(qb[i]), len(qphys), len(qb[i + 1]))
        if np.dtype(dtype).kind == "c":
            a = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
        else:
            a = rng.standard_normal(shape)
        a = a * block_mask(qb[i], qphys, qb[i + 1])
        As.append(np.asarray(a, dtype=dtype))
    return As, qb


def mps_charges(ql, qphys, qr):
    return (np.asarray(ql, np.int32), np.asarray(qphys, np.int32), np.asarray(qr, np.int32))


def sector_dims(q):
    """(charges, sizes) of a sorted charge array."""
    u, c = np.unique(np.asarray(q), return_counts=True)
    return u, c


def channel_charges(W, qphys):
    """U(1) charges of the virtual channels of a finite MPO with charge-definite channels
    (the charge labels TensorKit's graded MPO spaces carry).  A nonzero W[a, s, t, c] (s the
    bra, t the ket physical index) moves q_s - q_t into the channel: q_c = q_a + q_s - q_t.
    The boundary channels carry 0; the rule is applied in both directions until no label
    changes, and a channel no nonzero entry links to a labelled one carries 0 (its operator
    blocks vanish).  Returns L + 1 int32 arrays, array b for the bond left of site b; raises
    ValueError when two entries give one channel different charges."""
    qp = np.asarray(qphys, dtype=np.int64)
    unset = np.iinfo(np.int64).min
    n = len(W)
    q = [np.full(W[0].shape[0], unset, dtype=np.int64)]
    q += [np.full(w.shape[3], unset, dtype=np.int64) for w in W]
    q[0][:] = 0
    q[n][:] = 0
    links = []
    for w in W:
        nz = np.argwhere(np.asarray(w) != 0)
        dq = qp[nz[:, 1]] - qp[nz[:, 2]]
        links.append(np.unique(np.stack([nz[:, 0], nz[:, 3], dq], axis=1), axis=0))
    changed = True
    while changed:
        changed = False
        for i, trip in enumerate(links):
            for a, c, dq in trip.tolist():
                qa, qc = q[i][a], q[i + 1][c]
                if qa != unset and qc == unset:
                    q[i + 1][c] = qa + dq
                    changed = True
                elif qc != unset and qa == unset:
                    q[i][a] = qc - dq
                    changed = True
                elif qa != unset and qa + dq != qc:
                    raise ValueError(f"MPO channel {c} right of site {i} has no definite charge")
    return [np.where(x == unset, 0, x).astype(np.int32) for x in q]
