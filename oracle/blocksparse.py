"""U(1) block-sparse restatement of the two-site effective Hamiltonian and of the MPO transfer
(oracle; test infrastructure and the CPU arm of the benchmark).

TensorKit stores a U(1)-symmetric TensorMap as one dense block per coupled charge and runs
every `@plansor` contraction block by block.  Here tensors stay in the charge-sorted dense
embedding used everywhere else in the oracle (legs sorted by charge, exact zeros outside
the charge-conserving blocks), and every contraction is evaluated as TensorKit would: only
over the charge sectors that conserve charge, as dense GEMMs on contiguous slices of the
embedding.  Results equal the dense oracle (`oracle.derivatives`) to rounding; the work is
the block-sparse work.

Restated algorithms:
  * transfer_left / transfer_right(v, O, A, Ab)  -- src/transfermatrix/transfer.jl:125-130
  * JordanMPO_AC2_Hamiltonian matvec with the prepared terms
    (src/algorithms/derivatives/hamiltonian_derivatives.jl:272-500): the terms are built
    by `oracle.derivatives.JordanAC2` (same prepare folds); CA, AB, IC, BE and the
    continuing-continuing AA term run blockwise.  The AA term is evaluated in the order
    x.GR -> (W1 W2 mix) -> GL.(.) -- the same linear map as the prepared L.x.R form of
    mpo_derivatives.jl:233-288 with d times fewer flops (the cheaper order for a CPU).

Channel charges: an MPO channel carries the charge it adds to a bond.  Left environments
satisfy GL[a, w, a'] != 0 only if q_a - q_a' = dq[w]; the charges of the channels between
sites follow from the MPO alone, dq'[v] = dq[w] + q_s - q_t for W[w, s, t, v] != 0, starting
from the one-channel left boundary (dq = 0).  Right environments GR[b', w, b] are nonzero only
if q_b - q_b' = dq[w] (the same charges).
"""
import numpy as np

from . import derivatives as odv


def sector_slices(q):
    """charge -> slice of a charge-sorted leg."""
    q = np.asarray(q)
    assert np.all(np.diff(q) >= 0), "legs must be sorted by charge"
    out = {}
    if q.size == 0:
        return out
    cuts = np.flatnonzero(np.diff(q)) + 1
    starts = np.concatenate([[0], cuts])
    stops = np.concatenate([cuts, [q.size]])
    for a, b in zip(starts, stops):
        out[int(q[a])] = slice(int(a), int(b))
    return out


def mpo_channel_charges(Ws, qp):
    """Charges of the MPO channels on every bond of the chain: dq[i] for the left channels of
    site i (dq[0] = [0]); dq[i+1][v] = dq[i][w] + q_s - q_t over the nonzero W[i][w, s, t, v]."""
    qp = np.asarray(qp)
    out = [np.zeros(1, dtype=np.int64)]
    for W in Ws:
        wl, d, _, wr = W.shape
        cur = out[-1]
        nxt = np.full(wr, np.iinfo(np.int64).min, dtype=np.int64)
        w, s, t, v = np.nonzero(W)
        keep = _has(cur[w])  # channels that carry no charge (all-zero) pass nothing on
        w, s, t, v = w[keep], s[keep], t[keep], v[keep]
        vals = cur[w] + qp[s] - qp[t]
        for vv, val in zip(v, vals):
            if nxt[vv] == np.iinfo(np.int64).min:
                nxt[vv] = val
            else:
                assert nxt[vv] == val, "the MPO does not conserve the physical charges"
        out.append(nxt)
    return out


def _has(dq):
    return dq != np.iinfo(np.int64).min


def transfer_left(GL, W, A, ql, qp, qr, dq):
    """GL'[a, v, b] = GL[p, w, q] A[q, t, b] W[w, s, t, v] conj(A[p, s, a])  (transfer.jl:
    125-127) blockwise; ql / qr: charges of A's left / right bond, dq: channel charges of
    GL (left channels of W).  Returns GL' and the channel charges of its channels."""
    Dl, wl, _ = GL.shape
    d, wr, Dr = W.shape[1], W.shape[3], A.shape[2]
    qp = np.asarray(qp)
    dq_out = (np.full(wr, np.iinfo(np.int64).min, dtype=np.int64))
    w_, s_, t_, v_ = np.nonzero(W)
    for w, s, t, v in zip(w_, s_, t_, v_):
        if _has(dq[w]):
            dq_out[v] = dq[w] + qp[s] - qp[t]
    SL, SR = sector_slices(ql), sector_slices(qr)
    dt = np.result_type(GL.dtype, W.dtype, A.dtype)
    # T[(w, t)][kappa] = GL[P(kappa + dq_w), w, Q(kappa)] @ A[Q(kappa), t, B(kappa + q_t)]
    T = {}
    for w in range(wl):
        if not _has(dq[w]):
            continue
        for t in range(d):
            for kappa, Q in SL.items():
                P = SL.get(kappa + int(dq[w]))
                B = SR.get(kappa + int(qp[t]))
                if P is None or B is None:
                    continue
                T[(w, t, kappa)] = GL[P, w, Q] @ A[Q, t, B]
    out = np.zeros((Dr, wr, Dr), dtype=dt)
    # GL'[A(alpha), v, B(alpha - dq_v)] += sum_s A[P(alpha - q_s), s, A(alpha)]^H
    #                                      (sum_{w, t} W[w, s, t, v] T[(w, t, kappa)])
    by_vs = {}
    for w, s, t, v in zip(w_, s_, t_, v_):
        by_vs.setdefault((int(v), int(s)), []).append((int(w), int(t), W[w, s, t, v]))
    for (v, s), entries in by_vs.items():
        if not _has(dq_out[v]):
            continue
        for alpha, Aa in SR.items():
            pi = alpha - int(qp[s])
            P = SL.get(pi)
            B = SR.get(alpha - int(dq_out[v]))
            if P is None or B is None:
                continue
            Z = None
            for w, t, c in entries:
                blk = T.get((w, t, pi - int(dq[w])))
                if blk is None:
                    continue
                Z = c * blk if Z is None else Z + c * blk
            if Z is not None:
                out[Aa, v, B] += A[P, s, Aa].conj().T @ Z
    return out, dq_out


def transfer_right(GR, W, A, ql, qp, qr, dq):
    """GR'[a, w, b] = A[a, t, q] W[w, s, t, v] conj(A[b, s, r]) GR[q, v, r]  (transfer.jl:
    128-130) blockwise; dq: charges of W's left channels (those of GR'), GR[q, v, r] != 0
    only if q_r - q_q = dq_right[v] with dq_right[v] = dq[w] + q_s - q_t."""
    Dr, wr, _ = GR.shape
    d, wl, Dl = W.shape[1], W.shape[0], A.shape[0]
    qp = np.asarray(qp)
    SL, SR = sector_slices(ql), sector_slices(qr)
    dt = np.result_type(GR.dtype, W.dtype, A.dtype)
    w_, s_, t_, v_ = np.nonzero(W)
    dq_r = np.full(wr, np.iinfo(np.int64).min, dtype=np.int64)
    for w, s, t, v in zip(w_, s_, t_, v_):
        if _has(dq[w]):
            dq_r[v] = dq[w] + qp[s] - qp[t]
    # T[(v, t, ...)]: A[L(lam), t, Q(lam + q_t)] @ GR[Q(lam + q_t), v, R(lam + q_t + dq_v)]
    T = {}
    for v in range(wr):
        if not _has(dq_r[v]):
            continue
        for t in range(d):
            for lam, La in SL.items():
                Q = SR.get(lam + int(qp[t]))
                if Q is None:
                    continue
                Rr = SR.get(lam + int(qp[t]) + int(dq_r[v]))
                if Rr is None:
                    continue
                T[(v, t, lam)] = A[La, t, Q] @ GR[Q, v, Rr]
    out = np.zeros((Dl, wl, Dl), dtype=dt)
    by_ws = {}
    for w, s, t, v in zip(w_, s_, t_, v_):
        by_ws.setdefault((int(w), int(s)), []).append((int(v), int(t), W[w, s, t, v]))
    for (w, s), entries in by_ws.items():
        if not _has(dq[w]):
            continue
        # GR'[L(lam), w, L(lam + dq_w)] += (sum W T) @ conj(A[L(lam + dq_w), s, R(...)])^T
        for lam, La in SL.items():
            beta = lam + int(dq[w])
            Lb = SL.get(beta)
            Rr = SR.get(beta + int(qp[s]))
            if Lb is None or Rr is None:
                continue
            Z = None
            for v, t, c in entries:
                blk = T.get((v, t, lam))
                if blk is None:
                    continue
                Z = c * blk if Z is None else Z + c * blk
            if Z is not None:
                out[La, w, Lb] += Z @ A[Lb, s, Rr].conj().T
    return out


class JordanAC2U1:
    """JordanMPO_AC2_Hamiltonian of a U(1)-symmetric two-site problem, applied blockwise.

    GL, GR: environments (dense embedding); W1, W2: MPO tensors; ql, qr: charges of the outer
    bonds, qp: physical charges; dql: charges of GL's channels (W1's left channels), dqr:
    charges of W2's right channels (GR's)."""

    def __init__(self, GL, W1, W2, GR, ql, qp, qr, dql, dqr):
        self.op = odv.JordanAC2(GL, W1, W2, GR)
        self.ql, self.qp, self.qr = np.asarray(ql), np.asarray(qp), np.asarray(qr)
        self.SL, self.SR = sector_slices(ql), sector_slices(qr)
        self.d = len(qp)
        self.dtype = self.op.dtype
        t = self.op.t
        self.aa = None
        if t["AA"] is not None:
            GL2r, A1c, A2c, GR2c = t["AA"]
            A1, _, _, _ = odv.jordan_blocks(W1)
            A2, _, _, _ = odv.jordan_blocks(W2)
            rows, mids, cols = odv.connected_channels(A1, A2)
            dq_rows = np.asarray(dql)[1:-1][rows]
            dq_cols = np.asarray(dqr)[1:-1][cols]
            # coef[c, s1, s2, s1', s2', c'] = sum_m A1c[c, s1, s1', m] A2c[m, s2, s2', c']
            coef = np.einsum("cswm,mtuk->cstwuk", A1c, A2c, optimize=True)
            ent = {}
            for c, s1, s2, u1, u2, k in zip(*np.nonzero(coef)):
                ent.setdefault((int(c), int(s1), int(s2)), []).append(
                    (int(u1), int(u2), int(k), coef[c, s1, s2, u1, u2, k]))
            self.aa = (GL2r, GR2c, dq_rows, dq_cols, ent)
        self.mask = self._mask()

    def _mask(self):
        """Charge-allowed entries of x[l, s1, r, s2]: q_l + q_s1 + q_s2 = q_r."""
        ql, qp, qr = self.ql, self.qp, self.qr
        return (ql[:, None, None, None] + qp[None, :, None, None] + qp[None, None, None, :]
                == qr[None, None, :, None])

    # ------------------------------------------------------------- blockwise terms
    def _ca(self, x, CA, y):
        """y[a, p, b, r] += x[a, u, q, v] CA[p, r, b, u, v, q] per l-sector."""
        d, qp, SR = self.d, self.qp, self.SR
        for alpha, La in self.SL.items():
            kin = [(u, v, SR.get(alpha + int(qp[u]) + int(qp[v]))) for u in range(d) for v in range(d)]
            kin = [k for k in kin if k[2] is not None]
            out = [(p, r, SR.get(alpha + int(qp[p]) + int(qp[r]))) for p in range(d) for r in range(d)]
            out = [o for o in out if o[2] is not None]
            if not kin or not out:
                continue
            X = np.hstack([x[La, u, Q, v] for u, v, Q in kin])
            M = np.vstack([np.hstack([CA[p, r, B, u, v, Q].T for p, r, B in out])
                           for u, v, Q in kin])
            Y = X @ M
            o = 0
            for p, r, B in out:
                n = B.stop - B.start
                y[La, p, B, r] += Y[:, o:o + n]
                o += n

    def _ab(self, x, AB, y):
        """y[a, p, b, r] += AB[a, p, r, l, u, v] x[l, u, b, v] per r-sector."""
        d, qp, SL = self.d, self.qp, self.SL
        for beta, Rb in self.SR.items():
            kin = [(u, v, SL.get(beta - int(qp[u]) - int(qp[v]))) for u in range(d) for v in range(d)]
            kin = [k for k in kin if k[2] is not None]
            out = [(p, r, SL.get(beta - int(qp[p]) - int(qp[r]))) for p in range(d) for r in range(d)]
            out = [o for o in out if o[2] is not None]
            if not kin or not out:
                continue
            X = np.vstack([x[Ll, u, Rb, v] for u, v, Ll in kin])
            M = np.vstack([np.hstack([AB[La, p, r, Ll, u, v] for u, v, Ll in kin])
                           for p, r, La in out])
            Y = M @ X
            o = 0
            for p, r, La in out:
                n = La.stop - La.start
                y[La, p, Rb, r] += Y[o:o + n]
                o += n

    def _ic(self, x, IC, y):
        """y[a, p, b, r] += x[a, p, q, u] IC[r, b, u, q] per label mu = q_a + q_p."""
        d, qp, SL, SR = self.d, self.qp, self.SL, self.SR
        labels = {int(a) + int(b) for a in SL for b in qp}
        for mu in labels:
            rows = [(p, SL.get(mu - int(qp[p]))) for p in range(d)]
            rows = [r for r in rows if r[1] is not None]
            kin = [(u, SR.get(mu + int(qp[u]))) for u in range(d)]
            kin = [k for k in kin if k[1] is not None]
            out = [(r, SR.get(mu + int(qp[r]))) for r in range(d)]
            out = [o for o in out if o[1] is not None]
            if not rows or not kin or not out:
                continue
            X = np.vstack([np.hstack([x[La, p, Q, u] for u, Q in kin]) for p, La in rows])
            M = np.vstack([np.hstack([IC[r, B, u, Q].T for r, B in out]) for u, Q in kin])
            Y = X @ M
            i0 = 0
            for p, La in rows:
                m = La.stop - La.start
                j0 = 0
                for r, B in out:
                    n = B.stop - B.start
                    y[La, p, B, r] += Y[i0:i0 + m, j0:j0 + n]
                    j0 += n
                i0 += m

    def _be(self, x, BE, y):
        """y[a, p, b, r] += BE[a, p, l, u] x[l, u, b, r] per label mu = q_a + q_p."""
        d, qp, SL, SR = self.d, self.qp, self.SL, self.SR
        labels = {int(a) + int(b) for a in SL for b in qp}
        for mu in labels:
            rows = [(p, SL.get(mu - int(qp[p]))) for p in range(d)]
            rows = [r for r in rows if r[1] is not None]
            kin = [(u, SL.get(mu - int(qp[u]))) for u in range(d)]
            kin = [k for k in kin if k[1] is not None]
            out = [(r, SR.get(mu + int(qp[r]))) for r in range(d)]
            out = [o for o in out if o[1] is not None]
            if not rows or not kin or not out:
                continue
            X = np.vstack([np.hstack([x[Ll, u, B, r] for r, B in out]) for u, Ll in kin])
            M = np.vstack([np.hstack([BE[La, p, Ll, u] for u, Ll in kin]) for p, La in rows])
            Y = M @ X
            i0 = 0
            for p, La in rows:
                m = La.stop - La.start
                j0 = 0
                for r, B in out:
                    n = B.stop - B.start
                    y[La, p, B, r] += Y[i0:i0 + m, j0:j0 + n]
                    j0 += n
                i0 += m

    def _aa(self, x, y):
        """Continuing-continuing term: T1 = x . GR_c, the W1 W2 mix, y += GL_c . T2."""
        GL2r, GR2c, dq_rows, dq_cols, ent = self.aa
        d, qp, SL, SR = self.d, self.qp, self.SL, self.SR
        chc = GR2c.shape[1]
        # T1[(u1, u2, lam)] = x[L(lam), u1, R(kap), u2] @ [GR_c[R(kap), c', R(kap + dq_c')]]_c'
        T1 = {}
        for lam, Ll in SL.items():
            for u1 in range(d):
                for u2 in range(d):
                    kap = lam + int(qp[u1]) + int(qp[u2])
                    Q = SR.get(kap)
                    if Q is None:
                        continue
                    parts, offs = [], {}
                    o = 0
                    for k in range(chc):
                        Rr = SR.get(kap + int(dq_cols[k]))
                        if Rr is None:
                            continue
                        parts.append(GR2c[Q, k, Rr])
                        offs[k] = (o, o + Rr.stop - Rr.start)
                        o += Rr.stop - Rr.start
                    if parts:
                        T1[(u1, u2, lam)] = (x[Ll, u1, Q, u2] @ np.hstack(parts), offs)
        # y[L(al), s1, R(rho), s2] += sum_c GL_c[L(al), c, L(al - dq_c)] T2(c, s1, s2, al)
        chr_ = GL2r.shape[1]
        for al, La in SL.items():
            for s1 in range(d):
                for s2 in range(d):
                    rho = al + int(qp[s1]) + int(qp[s2])
                    Rr = SR.get(rho)
                    if Rr is None:
                        continue
                    Gs, Ts = [], []
                    for c in range(chr_):
                        lam = al - int(dq_rows[c])
                        Ll = SL.get(lam)
                        if Ll is None:
                            continue
                        Z = None
                        for u1, u2, k, cf in ent.get((c, s1, s2), ()):
                            blk = T1.get((u1, u2, lam))
                            if blk is None or k not in blk[1]:
                                continue
                            a, b = blk[1][k]
                            piece = cf * blk[0][:, a:b]
                            Z = piece if Z is None else Z + piece
                        if Z is not None:
                            Gs.append(GL2r[La, c, Ll])
                            Ts.append(Z)
                    if Gs:
                        y[La, s1, Rr, s2] += np.hstack(Gs) @ np.vstack(Ts)

    def __call__(self, x):
        t = self.op.t
        x = np.asarray(x)
        y = np.zeros(x.shape, dtype=np.result_type(x.dtype, self.dtype))
        if self.aa is not None:
            self._aa(x, y)
        if t["CA"] is not None:
            self._ca(x, t["CA"], y)
        if t["AB"] is not None:
            self._ab(x, t["AB"], y)
        if t["IC"] is not None:
            self._ic(x, t["IC"], y)
        if t["BE"] is not None:
            self._be(x, t["BE"], y)
        # the cheap leftovers (only when no GEMM term absorbed them): elementwise
        if t["II"] is not None:
            y += np.einsum("apqr,bq->apbr", x, t["II"], optimize=True)
        if t["ID"] is not None:
            y += np.einsum("apbu,ru->apbr", x, t["ID"], optimize=True)
        if t["CB"] is not None:
            y += np.einsum("aubv,pruv->apbr", x, t["CB"], optimize=True)
        if t["DE"] is not None:
            y += np.einsum("aubr,pu->apbr", x, t["DE"], optimize=True)
        if t["EE"] is not None:
            y += np.einsum("lpbr,al->apbr", x, t["EE"], optimize=True)
        return y * self.mask

    def block_flops(self):
        """2 x the multiply-adds of the blockwise GEMMs of one application: AA (x.GR_c and
        GL_c.T2), CA, AB, IC, BE -- the count a blockwise library executes."""
        d, qp, SL, SR = self.d, self.qp, self.SL, self.SR
        sz = lambda S, q: (S[q].stop - S[q].start) if q in S else 0
        t = self.op.t
        macs = 0
        if self.aa is not None:
            GL2r, GR2c, dq_rows, dq_cols, _ = self.aa
            for lam in SL:
                for u1 in range(d):
                    for u2 in range(d):
                        kap = lam + int(qp[u1]) + int(qp[u2])
                        n = sum(sz(SR, kap + int(q)) for q in dq_cols)
                        macs += sz(SL, lam) * sz(SR, kap) * n
            for al in SL:
                for s1 in range(d):
                    for s2 in range(d):
                        rho = al + int(qp[s1]) + int(qp[s2])
                        k = sum(sz(SL, al - int(q)) for q in dq_rows)
                        macs += sz(SL, al) * k * sz(SR, rho)
        if t["CA"] is not None:
            for al in SL:
                k = sum(sz(SR, al + int(qp[u]) + int(qp[v])) for u in range(d) for v in range(d))
                macs += sz(SL, al) * k * k
        if t["AB"] is not None:
            for be in SR:
                k = sum(sz(SL, be - int(qp[u]) - int(qp[v])) for u in range(d) for v in range(d))
                macs += k * k * sz(SR, be)
        for key in ("IC", "BE"):
            if t[key] is not None:
                for mu in {int(a) + int(b) for a in SL for b in qp}:
                    m = sum(sz(SL, mu - int(qp[p])) for p in range(d))
                    n = sum(sz(SR, mu + int(qp[r])) for r in range(d))
                    k = n if key == "IC" else m
                    macs += m * k * n
        return 2.0 * macs


# ---------------------------------------------------------------- environments and DMRG2

class FiniteEnvironmentsU1:
    """Lazy GL/GR cache of a U(1) FiniteMPS (oracle.mps.FiniteMPS with qb, qp), keyed on the
    identity of AL/AR (finite_envs.jl:110-151), built with the blockwise transfers.
    keep_newest: keep only the most recent environment per side (large D x w)."""

    def __init__(self, psi, H, keep_newest=False):
        L = len(psi)
        dt = np.result_type(psi.dtype, H.dtype)
        self.H = H
        self.dq = mpo_channel_charges([H[i] for i in range(L)], psi.qp)
        self.GL = [None] * (L + 1)
        self.GR = [None] * (L + 1)
        self.GL[0] = np.ones((1, 1, 1), dtype=dt)
        self.GR[L - 1] = np.ones((1, 1, 1), dtype=dt)
        self.ldep = [None] * L
        self.rdep = [None] * L
        self.keep_newest = keep_newest

    def leftenv(self, i, psi):
        first = next((j for j in range(i) if psi.AL[j] is not self.ldep[j]), i)
        if first == i and self.GL[i] is not None:
            return self.GL[i]
        start = max(k for k in range(first + 1) if self.GL[k] is not None)
        for j in range(start, i):
            self.GL[j + 1], _ = transfer_left(self.GL[j], self.H[j], psi.AL[j], psi.qb[j],
                                              psi.qp, psi.qb[j + 1], self.dq[j])
            self.ldep[j] = psi.AL[j]
            if self.keep_newest and j >= 1:
                self.GL[j] = None
        return self.GL[i]

    def rightenv(self, i, psi):
        L = len(psi)
        first = next((j for j in range(L - 1, i, -1) if psi.AR[j] is not self.rdep[j]), i)
        if first == i and self.GR[i] is not None:
            return self.GR[i]
        start = min(k for k in range(first, L) if self.GR[k] is not None)
        for j in range(start, i, -1):
            self.GR[j - 1] = transfer_right(self.GR[j], self.H[j], psi.AR[j], psi.qb[j],
                                            psi.qp, psi.qb[j + 1], self.dq[j])
            self.rdep[j] = psi.AR[j]
            if self.keep_newest and j <= L - 2:
                self.GR[j] = None
        return self.GR[i]


def ac2_hamiltonian(pos, psi, H, envs):
    return JordanAC2U1(envs.leftenv(pos, psi), H[pos], H[pos + 1], envs.rightenv(pos + 1, psi),
                       psi.qb[pos], psi.qp, psi.qb[pos + 2], envs.dq[pos], envs.dq[pos + 2])


def dmrg2_local_update(pos, right, psi, H, alg, envs, eps_global, eps_trunc, decay_rate, stats):
    """local_update!(..., ::DMRG2) (dmrg.jl:211-244) with block-sparse contractions: the
    Lanczos vectors hold only the charge-allowed entries of the two-site tensor (as a
    symmetric TensorMap does), the truncated SVD acts block by block."""
    from .krylov import lanczos_eigsolve
    from .mps import project_complement
    from .u1 import fuse, svd_trunc_u1
    Heff = ac2_hamiltonian(pos, psi, H, envs)
    if right:
        ac2 = np.einsum("asm,mtb->asbt", psi.ac(pos), psi.AR[pos + 1])
    else:
        ac2 = np.einsum("asm,mtb->asbt", psi.AL[pos], psi.ac(pos + 1))
    mask = Heff.mask
    shape = ac2.shape

    def apply(v):
        x = np.zeros(shape, dtype=np.result_type(v.dtype, Heff.dtype))
        x[mask] = v
        return Heff(x)[mask]

    y = Heff(ac2)
    stats["matvecs"] += 1
    y = y / np.linalg.norm(y)
    y = project_complement(y, psi.al(pos))
    eps_local = float(np.linalg.norm(y))
    kd, mi, tol = alg.alg_eigsolve.adapt(decay_rate, eps_local, eps_global, eps_trunc)
    val, newc, info = lanczos_eigsolve(apply, ac2[mask], krylovdim=kd, maxiter=mi, tol=tol,
                                       eager=alg.alg_eigsolve.eager)
    stats["matvecs"] += info.numops
    new = np.zeros(shape, dtype=newc.dtype)
    new[mask] = newc
    Dl, d1, Dr, d2 = shape
    M = new.reshape(Dl * d1, Dr * d2, order="F")
    qcol = (np.asarray(psi.qb[pos + 2])[:, None] - np.asarray(psi.qp)[None, :]).reshape(
        -1, order="F")
    U, S, Vh, qk, eps_tr = svd_trunc_u1(M, fuse(psi.qb[pos], psi.qp), qcol, alg.maxdim,
                                        alg.cutoff)
    psi.qb[pos + 1] = qk
    S = S / np.linalg.norm(S)
    k = S.size
    psi.AL[pos] = np.ascontiguousarray(U.reshape(Dl, d1, k, order="F").astype(psi.dtype))
    psi.AR[pos + 1] = np.ascontiguousarray(
        np.transpose(Vh.reshape(k, Dr, d2, order="F"), (0, 2, 1)).astype(psi.dtype))
    psi.C[pos + 1] = np.diag(S).astype(psi.dtype)
    psi.center = pos + 1
    decay = min(max((info.normres / eps_local) ** (1 / max(1, info.numops)), 1e-3), 0.999) \
        if eps_local > 0 else 0.999
    stats["block_flops"] = stats.get("block_flops", 0.0) + Heff.block_flops() * (info.numops + 1)
    return eps_local, eps_tr, decay, val


def canonical_u1(As, qb, qp, center):
    """FiniteMPS(As; normalize) (finitemps.jl:229-250) for a U(1) state, blockwise: a positive
    QR sweep left to right (oracle.u1.left_orth_u1 per charge block, R absorbed into the next
    tensor block by block), then positive LQ moves right to left down to the centre bond
    `center`.  Returns an oracle.mps.FiniteMPS with bond charges."""
    from .mps import FiniteMPS
    from .u1 import fuse, left_orth_u1, right_orth_u1
    L = len(As)
    qp = np.asarray(qp, np.int32)
    qb = [np.asarray(q, np.int32) for q in qb]
    A = [a.copy() for a in As]
    AL = [None] * L
    AR = [None] * L
    C = [None] * (L + 1)
    R = None
    for i in range(L):
        Dl, d, Dr = A[i].shape
        Q, R, qk = left_orth_u1(A[i].reshape(Dl * d, Dr, order="F"), fuse(qb[i], qp), qb[i + 1])
        AL[i] = Q.reshape(Dl, d, Q.shape[1], order="F")
        R = R / np.linalg.norm(R)
        if i < L - 1:
            # a sector with fewer rows than columns shrinks the bond (as in the dense sweep)
            A[i + 1] = _front_u1(R, A[i + 1], qk, qb[i + 1], qp, qb[i + 2])
        qb[i + 1] = qk
    C[L] = R
    X, qx = R, qb[L]
    for i in range(L - 1, center - 1, -1):
        a = _tail_u1(AL[i], X, qb[i], qp, qb[i + 1], qx)
        qb[i + 1] = qx
        Dl, d, Dr = a.shape
        qcol = (qb[i + 1][None, :] - qp[:, None]).reshape(-1, order="F")
        Lm, Q, qk = right_orth_u1(a.reshape(Dl, d * Dr, order="F"), qb[i], qcol)
        AR[i] = Q.reshape(Q.shape[0], d, Dr, order="F")
        C[i] = Lm
        # a sector with fewer columns than rows shrinks the bond (the new charges are qk)
        X, qx = Lm, qk
    qb[center] = qx
    return FiniteMPS(AL, AR, C, center=center, qb=qb, qp=qp)


def _front_u1(R, A, qk, ql, qp, qr):
    """R[k, l] A[l, s, r] for a charge-conserving R (q_k = q_l), block by block."""
    SK, SL, SR = sector_slices(qk), sector_slices(ql), sector_slices(qr)
    out = np.zeros((R.shape[0],) + A.shape[1:], dtype=np.result_type(R.dtype, A.dtype))
    for q, Sk in SK.items():
        Sq = SL.get(q)
        if Sq is None:
            continue
        for s in range(A.shape[1]):
            Sr = SR.get(q + int(qp[s]))
            if Sr is not None:
                out[Sk, s, Sr] = R[Sk, Sq] @ A[Sq, s, Sr]
    return out


def _tail_u1(A, X, ql, qp, qr, qk):
    """A[l, s, r] X[r, k] for a charge-conserving X (q_r = q_k), block by block."""
    SL, SR, SK = sector_slices(ql), sector_slices(qr), sector_slices(qk)
    out = np.zeros(A.shape[:2] + (X.shape[1],), dtype=np.result_type(A.dtype, X.dtype))
    for q, Sq in SL.items():
        for s in range(A.shape[1]):
            Sr = SR.get(q + int(qp[s]))
            Sk = SK.get(q + int(qp[s]))
            if Sr is not None and Sk is not None:
                out[Sq, s, Sk] = A[Sq, s, Sr] @ X[Sr, Sk]
    return out
