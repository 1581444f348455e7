"""Device-resident FiniteMPS and FiniteEnvironments.

  FiniteMPS(f, elt, P, maxV) + QR normalisation sweep -- src/states/finitemps.jl:229-282
  AC2(psi, site; kind)                                 -- src/states/finitemps.jl:376-385
  left_gauge / right_gauge / gauge2!                   -- src/states/orthoview.jl:322-420
  FiniteEnvironments leftenv / rightenv                -- src/environments/finite_envs.jl:31-49, 110-151

The state keeps AL/AR/C tensors in HBM with an explicit centre bond; environments
are recomputed lazily when the object identity of the AL/AR tensor they were built
from changes (the `===` dependency test of finite_envs.jl:111, 138).
"""
import ctypes

import numpy as np

from . import _lib as L
from .core import DeviceTensor, PackedTensor, context


def _wrap_out(ctx, *handles):
    return [DeviceTensor.wrap(ctx, h) for h in handles]


def _q(q):
    a = np.ascontiguousarray(q, dtype=np.int32)
    return a, a.ctypes.data_as(L.PI32)


def left_orth(AC):
    """AC = AL * C with a positive-diagonal QR (Householder(positive = true)); block by
    block when AC carries U(1) charges."""
    a, c = ctypes.c_void_p(), ctypes.c_void_p()
    if AC.charges is not None:
        (ql, pl), (qs, ps), (qr, pr) = (_q(x) for x in AC.charges)
        qk = np.zeros(min(AC.dims[0] * AC.dims[1], AC.dims[2]), dtype=np.int32)
        k = ctypes.c_int64()
        L.check(L.lib().gb_u1_left_orth(AC.ctx.handle, AC.handle, pl, ps, pr, ctypes.byref(a),
                                        ctypes.byref(c), qk.ctypes.data_as(L.PI32),
                                        ctypes.byref(k)))
        al, cc = _wrap_out(AC.ctx, a, c)
        qk = qk[:k.value].copy()
        al.charges, cc.charges = (ql, qs, qk), (qk, qr)
        return al, cc
    L.check(L.lib().gb_left_orth(AC.ctx.handle, AC.handle, ctypes.byref(a), ctypes.byref(c)))
    return tuple(_wrap_out(AC.ctx, a, c))


def right_orth(AC):
    """AC = C * AR with a positive-diagonal LQ (block by block for U(1) tensors)."""
    c, a = ctypes.c_void_p(), ctypes.c_void_p()
    if AC.charges is not None:
        (ql, pl), (qs, ps), (qr, pr) = (_q(x) for x in AC.charges)
        qk = np.zeros(min(AC.dims[0], AC.dims[1] * AC.dims[2]), dtype=np.int32)
        k = ctypes.c_int64()
        L.check(L.lib().gb_u1_right_orth(AC.ctx.handle, AC.handle, pl, ps, pr, ctypes.byref(c),
                                         ctypes.byref(a), qk.ctypes.data_as(L.PI32),
                                         ctypes.byref(k)))
        cc, ar = _wrap_out(AC.ctx, c, a)
        qk = qk[:k.value].copy()
        cc.charges, ar.charges = (ql, qk), (qk, qs, qr)
        return cc, ar
    L.check(L.lib().gb_right_orth(AC.ctx.handle, AC.handle, ctypes.byref(c), ctypes.byref(a)))
    return tuple(_wrap_out(AC.ctx, c, a))


def svd_trunc(AC2, maxdim=None, atol=0.0, normalize=True):
    """Truncated SVD of a two-site tensor -> (AL, S, AR, eps); per charge block, with the
    truncation global over blocks, for U(1) tensors."""
    a, s, r = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_void_p()
    eps = ctypes.c_double()
    if AC2.charges is not None:
        (ql, pl), (qs1, p1), (qr, pr), (qs2, p2) = (_q(x) for x in AC2.charges)
        Dl, d1, Dr, d2 = AC2.dims
        qk = np.zeros(min(Dl * d1, d2 * Dr), dtype=np.int32)
        k = ctypes.c_int64()
        L.check(L.lib().gb_u1_svd_trunc(AC2.ctx.handle, AC2.handle, pl, p1, pr, p2,
                                        int(maxdim or 0), float(atol), int(bool(normalize)),
                                        ctypes.byref(a), ctypes.byref(s), ctypes.byref(r),
                                        qk.ctypes.data_as(L.PI32), ctypes.byref(k),
                                        ctypes.byref(eps)))
        al, S, ar = _wrap_out(AC2.ctx, a, s, r)
        qk = qk[:k.value].copy()
        al.charges, S.charges, ar.charges = (ql, qs1, qk), (qk, qk), (qk, qs2, qr)
        return al, S, ar, eps.value
    L.check(L.lib().gb_svd_trunc(AC2.ctx.handle, AC2.handle, int(maxdim or 0), float(atol),
                                 int(bool(normalize)), ctypes.byref(a), ctypes.byref(s),
                                 ctypes.byref(r), ctypes.byref(eps)))
    al, S, ar = _wrap_out(AC2.ctx, a, s, r)
    return al, S, ar, eps.value


def _both(x, y):
    return x.charges is not None and y.charges is not None


def mul_front(C, A):
    out = DeviceTensor(A.ctx, L.GB_KIND_MPS, A.dtype, (C.dims[0], A.dims[1], A.dims[2]))
    L.check(L.lib().gb_mps_mul_front(A.ctx.handle, C.handle, A.handle, out.handle))
    if _both(C, A):
        out.charges = (C.charges[0], A.charges[1], A.charges[2])
    return out


def mul_tail(A, C):
    out = DeviceTensor(A.ctx, L.GB_KIND_MPS, A.dtype, (A.dims[0], A.dims[1], C.dims[1]))
    L.check(L.lib().gb_mps_mul_tail(A.ctx.handle, A.handle, C.handle, out.handle))
    if _both(A, C):
        out.charges = (A.charges[0], A.charges[1], C.charges[1])
    return out


def ac2_from(A, B):
    """AC2[l s1; r s2] = A[l s1; m] B[m s2; r]."""
    out = DeviceTensor(A.ctx, L.GB_KIND_AC2, A.dtype, (A.dims[0], A.dims[1], B.dims[2], B.dims[1]))
    L.check(L.lib().gb_mps_ac2(A.ctx.handle, A.handle, B.handle, out.handle))
    if _both(A, B):
        out.charges = (A.charges[0], A.charges[1], B.charges[2], B.charges[1])
    return out


def project_complement_(Y, X):
    L.check(L.lib().gb_project_complement(Y.ctx.handle, Y.handle, X.handle))
    return Y


def project_complement_right_(Y, X):
    """Y <- Y (1 - X' X) on the last two legs (X with orthonormal rows, e.g. AR)."""
    L.check(L.lib().gb_project_complement_right(Y.ctx.handle, Y.handle, X.handle))
    return Y


def mps_cat(A, B, leg, nb=None):
    """A (+) B along virtual leg 0 or 2 (catcodomain / catdomain); B = None appends `nb`
    zero rows / columns."""
    n = B.dims[leg] if B is not None else int(nb)
    dims = list(A.dims)
    dims[leg] += n
    out = DeviceTensor(A.ctx, L.GB_KIND_MPS, A.dtype, dims)
    L.check(L.lib().gb_mps_cat(A.ctx.handle, A.handle, B.handle if B is not None else None,
                               leg, out.handle))
    return out


def mps_permute(A, leg, perm, charges=None):
    """A with its bond leg 0 or 2 permuted, out[i] = A[perm[i]] along that leg
    (gb_mps_permute); `charges` of the result."""
    p = np.ascontiguousarray(perm, dtype=np.int64)
    out = DeviceTensor(A.ctx, L.GB_KIND_MPS, A.dtype, A.dims)
    L.check(L.lib().gb_mps_permute(A.ctx.handle, A.handle, int(leg),
                                   p.ctypes.data_as(L.PI64), out.handle))
    out.charges = charges
    return out


def perturb(env, W, AC, side, precision=L.GB_PREC_FP64):
    """The DMRG3S perturbation (gb_mps_perturb): side 0 with GL -> (Dl, d, Dr * wr),
    side 1 with GR -> (Dl * wl, d, Dr)."""
    Dl, d, Dr = AC.dims
    if side == 0:
        dims = (env.dims[0], d, Dr * W.dims[3])
    else:
        dims = (Dl * W.dims[0], d, env.dims[2])
    out = DeviceTensor(AC.ctx, L.GB_KIND_MPS, np.result_type(AC.dtype, env.dtype), dims)
    L.check(L.lib().gb_mps_perturb(AC.ctx.handle, side, env.handle, W.handle, AC.handle,
                                   precision, out.handle))
    return out


def bond_dims(L_, d, D):
    V = [1] * (L_ + 1)
    for k in range(1, L_):
        V[k] = min(V[k - 1] * d, D)
    for k in range(L_ - 1, 0, -1):
        V[k] = min(V[k], V[k + 1] * d)
    return V


def random_tensors(L_, d, D, seed, dtype=np.complex128):
    """Seeded i.i.d. normal entries (PCG64) on the full-rank virtual spaces."""
    rng = np.random.default_rng(seed)
    V = bond_dims(L_, d, D)
    out = []
    for i in range(L_):
        shape = (V[i], d, V[i + 1])
        if np.dtype(dtype).kind == "c":
            a = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
        else:
            a = rng.standard_normal(shape)
        out.append(np.asarray(a, dtype=dtype))
    return out


class FiniteMPS:
    """AL[i] valid for i < center, AR[i] for i >= center, C[center] the centre matrix."""

    def __init__(self, AL, AR, C, center):
        self.AL, self.AR, self.C, self.center = AL, AR, C, center

    def __len__(self):
        return len(self.AL)

    @property
    def ctx(self):
        return self.C[self.center].ctx

    @property
    def dtype(self):
        return self.C[self.center].dtype

    @classmethod
    def from_tensors(cls, As, ctx=None, normalize=True, center=0, charges=None):
        """FiniteMPS(As; normalize): positive-QR sweep left to right on the device, then
        LQ moves right to left down to the centre bond `center`.  `charges` =
        (bond charges [L+1 arrays], physical charges) makes it a U(1)-symmetric state
        (mpsgb.u1): the gauge steps then act per charge block."""
        ctx = ctx or context()
        n = len(As)
        A = [DeviceTensor.from_numpy(ctx, L.GB_KIND_MPS, a) for a in As]
        if charges is not None:
            qb, qp = charges
            for i, a in enumerate(A):
                a.charges = (np.asarray(qb[i], np.int32), np.asarray(qp, np.int32),
                             np.asarray(qb[i + 1], np.int32))
        AL = [None] * n
        C = [None] * (n + 1)
        R = None
        for i in range(n):
            q, R = left_orth(A[i])
            if normalize:
                R.scale_(1.0 / R.norm())
            AL[i] = q
            if i < n - 1:
                A[i + 1] = mul_front(R, A[i + 1])
        C[n] = R
        psi = cls(AL, [None] * n, C, n)
        psi.right_canonicalize(center)
        return psi

    @classmethod
    def random(cls, L_, d, D, seed, dtype=np.complex128, ctx=None):
        return cls.from_tensors(random_tensors(L_, d, D, seed, dtype), ctx)

    def right_canonicalize(self, stop=0):
        """Move the centre bond down to `stop` with positive LQ factorisations."""
        X = self.C[self.center]
        for i in range(self.center - 1, stop - 1, -1):
            A = mul_tail(self.AL[i], X)
            Lm, Q = right_orth(A)
            self.AR[i] = Q
            self.C[i] = Lm
            X = Lm
        self.center = stop
        return self

    def ac(self, i):
        """AC[i] for a centre bond at i or i+1, or the explicitly stored AC of site i."""
        if getattr(self, "ac_site", None) == i:
            return self.ac_tensor
        if self.center == i:
            return mul_front(self.C[i], self.AR[i])
        if self.center == i + 1:
            return mul_tail(self.AL[i], self.C[i + 1])
        raise ValueError(f"site {i} is not adjacent to the centre bond {self.center}")

    def al(self, i):
        if i < self.center:
            return self.AL[i]
        q, _ = left_orth(self.ac(i))
        return q

    def to_numpy(self):
        """Host copies (AL, AR, C, center) in reference layout."""
        f = lambda xs: [None if x is None else x.numpy() for x in xs]
        return f(self.AL), f(self.AR), f(self.C), self.center


class FiniteEnvironments:
    """Lazy GL/GR cache.  With `resident=False` only the most recently computed
    environment of each side stays in HBM (older ones are released and recomputed from
    the boundary when asked for again) -- the memory policy for large D x w, where all
    L environments do not fit on one device.  `keep_left` / `keep_right`: sites whose
    environments are never released (e.g. the right environments of a window of bonds a
    sweep is about to visit).  With `packed=True` every environment stays resident but only
    the newest (or last requested) one of each side is held dense: the others are
    tile-packed (gb_tensor_pack, exact), a tenth of the dense embedding of a U(1)
    environment, and unpacked when asked for again."""

    def __init__(self, psi, H, ctx=None, resident=True, keep_left=(), keep_right=(),
                 packed=False):
        self.packed = packed
        self.resident = resident or packed
        self.keep_left, self.keep_right = set(keep_left), set(keep_right)
        self.ctx = ctx or psi.ctx
        self.H = H
        n = len(psi)
        self.dtype = np.result_type(psi.dtype, H.dtype)
        one = np.ones((1, 1, 1), dtype=self.dtype)
        self.GL = [None] * (n + 1)
        self.GR = [None] * (n + 1)
        self.GL[0] = DeviceTensor.from_numpy(self.ctx, L.GB_KIND_GL, one)
        self.GR[n - 1] = DeviceTensor.from_numpy(self.ctx, L.GB_KIND_GR, one)
        self.ldep = [None] * n
        self.rdep = [None] * n
        self.precision = L.GB_PREC_FP64

    def _W(self):
        return self.H.device(self.ctx, self.dtype)

    def _dense(self, lst, i):
        """lst[i] as a dense tensor; with packing on, every other environment of that side
        (but the boundary ones) is packed."""
        t = lst[i]
        if not self.packed:
            return t
        if isinstance(t, PackedTensor):
            t = lst[i] = t.unpack()
        last = len(lst) - 1
        for k, o in enumerate(lst):
            if k != i and isinstance(o, DeviceTensor) and 0 < k < last and min(o.dims) > 1:
                lst[k] = PackedTensor(o)
        return t

    def leftenv(self, i, psi):
        """GL of site i, recomputed from the nearest valid environment below when an AL
        it depends on changed (by identity) or when it was released."""
        first = next((j for j in range(i) if psi.AL[j] is not self.ldep[j]), i)
        if first == i and self.GL[i] is not None:
            return self._dense(self.GL, i)
        start = max(k for k in range(first + 1) if self.GL[k] is not None)
        W = self._W()
        for j in range(start, i):
            self._dense(self.GL, j)
            A = psi.AL[j]
            out = DeviceTensor(self.ctx, L.GB_KIND_GL, self.dtype,
                               (A.dims[2], W[j].dims[3], A.dims[2]))
            L.check(L.lib().gb_env_transfer_left(self.ctx.handle, self.GL[j].handle,
                                                 W[j].handle, A.handle, A.handle,
                                                 self.precision, out.handle))
            self.GL[j + 1] = out
            self.ldep[j] = A
            if not self.resident and j >= 1 and j not in self.keep_left:
                self.GL[j] = None
        return self._dense(self.GL, i)

    def rightenv(self, i, psi):
        """GR of site i (everything right of i), recomputed from the nearest valid
        environment above when an AR it depends on changed or was released."""
        n = len(psi)
        first = next((j for j in range(n - 1, i, -1) if psi.AR[j] is not self.rdep[j]), i)
        if first == i and self.GR[i] is not None:
            return self._dense(self.GR, i)
        start = min(k for k in range(first, n) if self.GR[k] is not None)
        W = self._W()
        for j in range(start, i, -1):
            self._dense(self.GR, j)
            A = psi.AR[j]
            out = DeviceTensor(self.ctx, L.GB_KIND_GR, self.dtype,
                               (A.dims[0], W[j].dims[0], A.dims[0]))
            L.check(L.lib().gb_env_transfer_right(self.ctx.handle, self.GR[j].handle,
                                                  W[j].handle, A.handle, A.handle,
                                                  self.precision, out.handle))
            self.GR[j - 1] = out
            self.rdep[j] = A
            if not self.resident and j <= n - 2 and j not in self.keep_right:
                self.GR[j] = None
        return self._dense(self.GR, i)
