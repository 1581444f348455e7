"""MPOHamiltonian in Jordan block form, built from lattice terms.

Restates MPSKit's builder (src/operators/mpohamiltonian.jl:349-519 finite,
:521-641 infinite): terms are instantiated with identity strings between their sites
(`instantiate_operator`, :360-386), sorted by range, and every term gets its own
continuing channel on each bond it crosses (`_find_channel`, :408-416: the smallest
free channel label >= the incoming one).  Two-site operators are split by a truncated
SVD into a left isometry and a right factor (`decompose_localmpo`,
src/utility/utility.jl:54-66).  The result is stored densely over the channel sum
space, W[wl, s, s', wr], with channel 0 = "not started" and the last channel =
"finished" -- the JordanMPOTensor layout (src/operators/jordanmpotensor.jl:1-66)
flattened, which is also the GB_KIND_MPO format of the C ABI.
"""
import numpy as np

from . import _lib as L
from .core import DeviceTensor

_SX = np.array([[0, 1], [1, 0]], dtype=np.complex128) / 2
_SY = np.array([[0, -1j], [1j, 0]], dtype=np.complex128) / 2
_SZ = np.array([[1, 0], [0, -1]], dtype=np.complex128) / 2


def spin_half():
    """(Sx, Sy, Sz) = sigma/2."""
    return _SX.copy(), _SY.copy(), _SZ.copy()


def kron2(a, b):
    """Two-site operator O[s1, s2; s1', s2'] = a[s1, s1'] b[s2, s2']."""
    return np.einsum("ik,jl->ijkl", a, b)


def _as(a, dtype):
    a = np.asarray(a)
    if np.dtype(dtype).kind == "f":
        if np.abs(a.imag).max(initial=0.0) > 1e-14:
            raise ValueError("operator is not real")
        return np.ascontiguousarray(a.real, dtype=np.float64)
    return np.ascontiguousarray(a, dtype=np.complex128)


def split_two_site(op, atol=None, qphys=None):
    """op[s1,s2,s1',s2'] = sum_k L[s1,s1',k] R[k,s2,s2'] with an isometric left factor.

    With physical charges `qphys` (U(1)), the split is done per charge transfer
    delta = q(s1) - q(s1'), so that every channel carries a definite charge (the channel
    spaces of a symmetric MPO, src/operators/mpohamiltonian.jl:439-519, are graded the same
    way); `op` must conserve charge."""
    d1, d2 = op.shape[0], op.shape[1]
    atol = np.finfo(np.float64).eps ** 0.75 if atol is None else atol
    M = op.transpose(0, 2, 1, 3).reshape(d1 * d1, d2 * d2)
    if qphys is None:
        U, S, Vh = np.linalg.svd(M, full_matrices=False)
        r = int((S > atol).sum())
        left = U[:, :r].reshape(d1, d1, r)
        right = (S[:r, None] * Vh[:r]).reshape(r, d2, d2)
        return left.astype(op.dtype), right.astype(op.dtype)
    q = np.asarray(qphys)
    dqr = (q[:d1, None] - q[None, :d1]).reshape(-1)   # row s1*d1 + s1'
    dqc = (q[:d2, None] - q[None, :d2]).reshape(-1)   # col s2*d2 + s2'
    lefts, rights = [], []
    rest = M.copy()
    for delta in sorted(set(dqr.tolist())):
        rows = np.nonzero(dqr == delta)[0]
        cols = np.nonzero(dqc == -delta)[0]
        if rows.size == 0 or cols.size == 0:
            continue
        blk = M[np.ix_(rows, cols)]
        rest[np.ix_(rows, cols)] = 0
        U, S, Vh = np.linalg.svd(blk, full_matrices=False)
        for k in range(int((S > atol).sum())):
            lv = np.zeros(d1 * d1, dtype=M.dtype)
            rv = np.zeros(d2 * d2, dtype=M.dtype)
            lv[rows] = U[:, k]
            rv[cols] = S[k] * Vh[k]
            lefts.append(lv)
            rights.append(rv)
    if np.abs(rest).max(initial=0.0) > atol:
        raise ValueError("two-site operator does not conserve the given charges")
    left = np.stack(lefts, axis=1).reshape(d1, d1, len(lefts))
    right = np.stack(rights, axis=0).reshape(len(rights), d2, d2)
    return left.astype(op.dtype), right.astype(op.dtype)


class MPOHamiltonian:
    """Dense Jordan-form MPO.  `W[i]` has shape (wl, d, d, wr)."""

    def __init__(self, W, finite=True, chans=None):
        self.W = list(W)
        self.finite = finite
        # chans[i]: dimensions of the channel blocks (sum-space components) of the bond
        # left of site i; the blocks are the "levels" of the infinite environments
        self.chans = chans
        self._dev = {}

    def __len__(self):
        return len(self.W)

    def __getitem__(self, i):
        return self.W[i % len(self.W)]

    @property
    def dtype(self):
        return self.W[0].dtype

    def widths(self):
        return [w.shape[3] for w in self.W]

    # ---------------------------------------------------------------- linear algebra
    # (mpohamiltonian.jl:741-786, 815-820: the Jordan blocks of a sum are A = A1 (+) A2 on
    # the continuing channels, B and C stacked along them, D = D1 + D2; the identity corners
    # stay single.  A scalar multiplies every term once: the C and D blocks.)
    def __add__(self, other):
        if np.isscalar(other) or isinstance(other, (list, tuple, np.ndarray)):
            return self._add_onsite(other)
        if not isinstance(other, MPOHamiltonian):
            return NotImplemented
        if len(self) != len(other) or self.finite != other.finite:
            raise ValueError("sum of MPOHamiltonians of different lengths or kinds")
        W = [_jordan_sum(a, b) for a, b in zip(self.W, other.W)]
        chans = None
        if self.chans is not None and other.chans is not None:
            chans = [list(a) if len(a) == 1
                     else [a[0]] + list(a[1:-1]) + list(b[1:-1]) + [a[-1]]
                     for a, b in zip(self.chans, other.chans)]
        return MPOHamiltonian(W, finite=self.finite, chans=chans)

    __radd__ = __add__

    def _add_onsite(self, lams):
        """H + lambdas (mpohamiltonian.jl:788-813): lambda_i times the identity on site i,
        added to the D (start -> finish) block; a scalar applies to every site."""
        lams = np.broadcast_to(np.asarray(lams), (len(self),))
        W = []
        for w, lam in zip(self.W, lams):
            w = w.astype(np.result_type(w.dtype, np.asarray(lam).dtype), copy=True)
            w[0, :, :, w.shape[3] - 1] += lam * np.eye(w.shape[1], dtype=w.dtype)
            W.append(w)
        return MPOHamiltonian(W, finite=self.finite, chans=self.chans)

    def __mul__(self, lam):
        if isinstance(lam, MPOHamiltonian):
            return self._product(lam)
        if not np.isscalar(lam):
            return NotImplemented
        W = []
        for w in self.W:
            w = w.astype(np.result_type(w.dtype, np.asarray(lam).dtype), copy=True)
            first = 1 if w.shape[3] > 1 else 0   # the start column continues unscaled
            w[0, :, :, first:] *= lam
            W.append(w)
        return MPOHamiltonian(W, finite=self.finite, chans=self.chans)

    def __rmul__(self, lam):
        return self.__mul__(lam)

    def _product(self, other):
        """H1 * H2 (mpohamiltonian.jl:848-852, fuse_mul_mpo per site): the operator product
        (H1 H2)[s; s'] = sum_t H1[s; t] H2[t; s'] with the channel pairs (c1, c2) fused, c1
        major -- upper triangular again, start (start, start) first and finish (finish,
        finish) last."""
        if len(self) != len(other) or self.finite != other.finite:
            raise ValueError("product of MPOHamiltonians of different lengths or kinds")
        W = []
        for a, b in zip(self.W, other.W):
            # (a1, s, t, b1) x (a2, t, s', b2) -> (a1, a2, s, s', b1, b2)
            w = np.einsum("astb,ctud->acsubd", a, b)
            W.append(w.reshape(a.shape[0] * b.shape[0], a.shape[1], b.shape[2],
                               a.shape[3] * b.shape[3]))
        chans = None
        if self.chans is not None and other.chans is not None:
            chans = [[x * y for x in ca for y in cb] for ca, cb in zip(self.chans, other.chans)]
        return MPOHamiltonian(W, finite=self.finite, chans=chans)

    def __neg__(self):
        return self * -1.0

    def __sub__(self, other):
        if isinstance(other, MPOHamiltonian):
            return self + (-other)
        return self + (-np.asarray(other))

    def channel_charges(self, qphys):
        """U(1) charges of the channels on every bond (`u1.channel_charges`), cached per
        physical charge assignment."""
        from .u1 import channel_charges
        key = ("charges",) + tuple(int(x) for x in qphys)
        if key not in self._dev:
            self._dev[key] = channel_charges(self.W, qphys)
        return self._dev[key]

    def device(self, ctx, dtype=None):
        """GB_KIND_MPO tensors of every site (cached per context and dtype)."""
        dtype = np.dtype(dtype or self.dtype)
        key = (id(ctx), dtype.str)
        if key not in self._dev:
            self._dev[key] = [DeviceTensor.from_numpy(ctx, L.GB_KIND_MPO, w, dtype) for w in self.W]
        return self._dev[key]


def _jordan_sum(W1, W2):
    """The site tensor of H1 + H2 (one site of mpohamiltonian.jl:741-786): left channels
    [start, mid(H1), mid(H2), finish] (only [start] at a finite chain's first site), right
    channels likewise (only [finish] at its last site)."""
    wl1, d, _, wr1 = W1.shape
    wl2, wr2 = W2.shape[0], W2.shape[3]
    if (wl1 == 1) != (wl2 == 1) or (wr1 == 1) != (wr2 == 1) or W2.shape[1] != d:
        raise ValueError("sum of MPO site tensors of different boundary structure")
    lm1 = list(range(1, wl1 - 1)) if wl1 > 1 else []
    lm2 = list(range(1, wl2 - 1)) if wl2 > 1 else []
    rm1 = list(range(1, wr1 - 1)) if wr1 > 1 else []
    rm2 = list(range(1, wr2 - 1)) if wr2 > 1 else []
    nl = 1 if wl1 == 1 else 2 + len(lm1) + len(lm2)
    nr = 1 if wr1 == 1 else 2 + len(rm1) + len(rm2)

    def maps(wl, wr, lm, rm, loff, roff):
        Lm, Rm = {0: 0}, {wr - 1: nr - 1}
        if wl > 1:
            Lm[wl - 1] = nl - 1
        if wr > 1:
            Rm[0] = 0
        Lm.update({i: 1 + loff + k for k, i in enumerate(lm)})
        Rm.update({j: 1 + roff + k for k, j in enumerate(rm)})
        return Lm, Rm

    W = np.zeros((nl, d, d, nr), dtype=np.result_type(W1.dtype, W2.dtype))
    L1, R1 = maps(wl1, wr1, lm1, rm1, 0, 0)
    L2, R2 = maps(wl2, wr2, lm2, rm2, len(lm1), len(rm1))
    for i in range(wl1):
        for j in range(wr1):
            W[L1[i], :, :, R1[j]] += W1[i, :, :, j]
    for i in range(wl2):
        for j in range(wr2):
            start_start = wr2 > 1 and i == 0 and j == 0
            finish_finish = wl2 > 1 and i == wl2 - 1 and j == wr2 - 1
            if not (start_start or finish_finish):   # identity corners once
                W[L2[i], :, :, R2[j]] += W2[i, :, :, j]
    return W


def _site_pieces(sites, op, qphys=None):
    if len(sites) == 1:
        return [op.reshape(1, op.shape[0], op.shape[1], 1)]
    a, b = split_two_site(op, qphys=qphys)
    return [a.reshape(1, a.shape[0], a.shape[1], a.shape[2]),
            b.reshape(b.shape[0], b.shape[1], b.shape[2], 1)]


def _normalize_terms(terms, dtype, qphys=None):
    out = []
    for sites, op in terms:
        sites = tuple(int(s) for s in sites)
        op = _as(op, dtype)
        if len(sites) == 2 and sites[0] > sites[1]:
            sites = (sites[1], sites[0])
            op = op.transpose(1, 0, 3, 2)
        if len(sites) == 2 and sites[0] == sites[1]:
            raise ValueError("a two-site term needs two distinct sites")
        pieces = _site_pieces(sites, op, qphys)
        span = list(range(sites[0], sites[-1] + 1))
        chain = []
        it = iter(pieces)
        for s in span:
            chain.append(next(it) if s in sites else 1.0)
        out.append((span, chain))
    out.sort(key=lambda t: len(t[0]))
    return out


def _free_channel(used, start):
    c = max(start, 2)
    taken = set(used)
    while c in taken:
        c += 1
    return c


def _assign(terms, nsites, wrap):
    keys = [[] for _ in range(nsites)]
    ops = [[] for _ in range(nsites)]
    for span, chain in terms:
        incoming = 1
        for j, (site, piece) in enumerate(zip(span, chain)):
            s = site % nsites if wrap else site
            outgoing = 0 if j == len(chain) - 1 else _free_channel([k[1] for k in keys[s]], incoming)
            keys[s].append((incoming, outgoing))
            ops[s].append(piece)
            incoming = outgoing
    return keys, ops


def _fill(keys_s, ops_s, cl, cr, d, dtype, identity_corners):
    offl = np.concatenate([[0], np.cumsum(cl)]).astype(int)
    offr = np.concatenate([[0], np.cumsum(cr)]).astype(int)
    W = np.zeros((offl[-1], d, d, offr[-1]), dtype=dtype)
    nr, nc = len(cl), len(cr)
    if identity_corners:
        if nc > 1:
            W[0, :, :, 0] += np.eye(d)
        if nr > 1:
            W[offl[-2], :, :, offr[-2]] += np.eye(d)
    for (kl, kr), piece in zip(keys_s, ops_s):
        kr = nc if kr == 0 else kr
        rl = slice(offl[kl - 1], offl[kl])
        rr = slice(offr[kr - 1], offr[kr])
        if isinstance(piece, np.ndarray):
            W[rl, :, :, rr] += piece
        elif piece != 0:
            n = offl[kl] - offl[kl - 1]
            W[rl, :, :, rr] += piece * np.einsum("ab,st->astb", np.eye(n), np.eye(d))
    return W


def FiniteMPOHamiltonian(nsites, d, terms, dtype=np.complex128, qphys=None):
    """Jordan-form MPO of sum(terms) on an open chain of `nsites` sites of dimension d
    (`qphys`: U(1) charges of the physical basis, for charge-definite channels)."""
    terms = _normalize_terms(terms, dtype, qphys)
    keys, ops = _assign(terms, nsites, wrap=False)
    chans = [[1] for _ in range(nsites + 1)]
    for i in range(nsites - 1):
        n = max([k[1] for k in keys[i]] + [1]) + 1
        V = [1] * n
        if n > 2:
            for (kl, kr), piece in zip(keys[i], ops[i]):
                idx = n - 1 if kr == 0 else kr - 1
                V[idx] = piece.shape[3] if isinstance(piece, np.ndarray) else chans[i][kl - 1]
        chans[i + 1] = V
    W = [_fill(keys[i], ops[i], chans[i], chans[i + 1], d, np.dtype(dtype), True)
         for i in range(nsites)]
    return MPOHamiltonian(W, finite=True, chans=chans)


def InfiniteMPOHamiltonian(ncell, d, terms, dtype=np.complex128, qphys=None):
    """Jordan-form MPO of a translation-invariant sum of terms with unit cell `ncell`."""
    terms = _normalize_terms(terms, dtype, qphys)
    keys, ops = _assign(terms, ncell, wrap=True)
    n = max(max([k[1] for k in K] + [1]) + 1 for K in keys)
    V = [[None] * n for _ in range(ncell)]   # V[i] = channels right of site i
    for v in V:
        v[0] = 1
        v[-1] = 1
    for i in range(ncell):
        for (kl, kr), piece in zip(keys[i], ops[i]):
            if not isinstance(piece, np.ndarray):
                continue
            kr = n if kr == 0 else kr
            V[i - 1][kl - 1] = piece.shape[0]
            V[i][kr - 1] = piece.shape[3]
    changed = True
    while changed:
        changed = False
        for i in range(ncell):
            for (kl, kr), piece in zip(keys[i], ops[i]):
                if isinstance(piece, np.ndarray):
                    continue
                kr = n if kr == 0 else kr
                a, b = V[i - 1][kl - 1], V[i][kr - 1]
                if a is not None and b is None:
                    V[i][kr - 1] = a
                    changed = True
                elif a is None and b is not None:
                    V[i - 1][kl - 1] = b
                    changed = True
    V = [[1 if x is None else x for x in v] for v in V]
    W = [_fill(keys[i], ops[i], V[i - 1], V[i], d, np.dtype(dtype), True) for i in range(ncell)]
    return MPOHamiltonian(W, finite=False, chans=[V[i - 1] for i in range(ncell)] + [V[ncell - 1]])


# ------------------------------------------------------------------ models

# U(1) charges (2 Sz) of the spin-1/2 basis |up>, |down>
SPIN_HALF_CHARGES = np.array([1, -1], dtype=np.int32)


def heisenberg_XXX(L, J=1.0, dtype=np.complex128, infinite=False, u1=False):
    """J sum S_i . S_{i+1} for spin 1/2 (`u1`: channels of definite Sz transfer)."""
    sx, sy, sz = spin_half()
    h = J * (kron2(sx, sx) + kron2(sy, sy) + kron2(sz, sz))
    q = SPIN_HALF_CHARGES if u1 else None
    if infinite:
        return InfiniteMPOHamiltonian(L, 2, [((i, i + 1), h) for i in range(L)], dtype, q)
    return FiniteMPOHamiltonian(L, 2, [((i, i + 1), h) for i in range(L - 1)], dtype, q)


def xxz(L, Jxy=1.0, Jz=1.0, hz=0.0, dtype=np.complex128, infinite=False, u1=False,
        rotated=False):
    """sum Jxy (SxSx + SySy) + Jz SzSz - hz sum Sz.  rotated=True applies a rotation by pi
    about x on every other site (same spectrum; hz = 0 only): Jxy (SxSx - SySy) - Jz SzSz per
    bond, one-site translation invariant in the Neel phase.  It does not conserve Sz."""
    sx, sy, sz = spin_half()
    if rotated:
        if hz or u1:
            raise ValueError("rotated XXZ: no field and no U(1) charges")
        h = Jxy * (kron2(sx, sx) - kron2(sy, sy)) - Jz * kron2(sz, sz)
    else:
        h = Jxy * (kron2(sx, sx) + kron2(sy, sy)) + Jz * kron2(sz, sz)
    nb = L if infinite else L - 1
    terms = [((i, i + 1), h) for i in range(nb)]
    if hz:
        terms += [((i,), -hz * sz) for i in range(L)]
    build = InfiniteMPOHamiltonian if infinite else FiniteMPOHamiltonian
    return build(L, 2, terms, dtype, SPIN_HALF_CHARGES if u1 else None)


def transverse_field_ising(L, g=1.0, J=1.0, dtype=np.complex128, infinite=False):
    """-J sum Z Z - g sum X with Pauli X = 2Sx, Z Z = 4 Sz Sz."""
    sx, sy, sz = spin_half()
    nb = L if infinite else L - 1
    terms = [((i,), -g * 2 * sx) for i in range(L)]
    terms += [((i, i + 1), -J * 4 * kron2(sz, sz)) for i in range(nb)]
    build = InfiniteMPOHamiltonian if infinite else FiniteMPOHamiltonian
    return build(L, 2, terms, dtype)


def j1j2_cylinder(Lx, Ly, J1=1.0, J2=0.5, dtype=np.float64, u1=False):
    """J1-J2 Heisenberg on an Lx x Ly cylinder (periodic in y, open in x), snake-ordered."""
    def site(x, y):
        y %= Ly
        return x * Ly + (y if x % 2 == 0 else Ly - 1 - y)

    sx, sy, sz = spin_half()
    h = kron2(sx, sx) + kron2(sy, sy) + kron2(sz, sz)
    bonds = {}

    def add(a, b, J):
        if a != b:
            key = (min(a, b), max(a, b))
            bonds[key] = bonds.get(key, 0.0) + J

    for x in range(Lx):
        for y in range(Ly):
            if Ly > 2 or y + 1 < Ly:
                add(site(x, y), site(x, y + 1), J1)
            if x + 1 < Lx:
                add(site(x, y), site(x + 1, y), J1)
                add(site(x, y), site(x + 1, y + 1), J2)
                add(site(x, y), site(x + 1, y - 1), J2)
    terms = [((a, b), J * h) for (a, b), J in sorted(bonds.items())]
    return FiniteMPOHamiltonian(Lx * Ly, 2, terms, dtype, SPIN_HALF_CHARGES if u1 else None)
