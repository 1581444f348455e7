"""The Gram-matrix truncation (GB_SVD_GRAM) near its resolution floor.

Singular values taken as sqrt(eig(M^H M)) carry an absolute error of about
eps_mach * s_max^2 / s, so below ~1e-7 s_max they are rounding noise.  With a cutoff of
atol = 1e-10 (the configurations' trunctol) the kept rank and the discarded weight must
still be those of the SVD (src/states/orthoview.jl:405, svd_trunc with trunctol): the call
falls back to the SVD whenever a kept or the first discarded value lies below the floor.
Spectra are prescribed exactly (M = U diag(s) V^H with random orthonormal U, V)."""
import numpy as np
import pytest

import mpsgb
from mpsgb import u1 as HU
from mpsgb.operators import SPIN_HALF_CHARGES as QP
from oracle import mps as P
from oracle import u1 as U

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = mpsgb.context(0)
    yield c
    c.set_svd_method("gesvd")


def _orth(rng, n, k):
    q, _ = np.linalg.qr(rng.standard_normal((n, k)))
    return q


def _dense_ac2(rng, Dl, Dr, spectrum):
    m, n = 2 * Dl, 2 * Dr
    k = len(spectrum)
    M = _orth(rng, m, k) @ np.diag(spectrum) @ _orth(rng, n, k).T
    # device/TensorKit layout x[l s1; r s2]: rows (l, s1), columns (s2, r)
    return M.reshape(Dl, 2, 2, Dr, order="F").transpose(0, 1, 3, 2).copy(order="F"), M


def _is_diag(a):
    return np.count_nonzero(a - np.diag(np.diag(a))) == 0


@pytest.mark.parametrize("spread", ["deep", "benign"])
def test_dense_gram_truncation_matches_svd(ctx, spread):
    rng = np.random.default_rng(11)
    Dl, Dr = 40, 36
    # full rank (72 = min(2 Dl, 2 Dr)): a rank-deficient matrix has exact zeros, which the
    # Gram route sees as noise and hands to the SVD as well
    if spread == "deep":
        s = np.logspace(0, -12, 72)  # values in [1e-10, 1e-7] decide the rank at atol 1e-10
    else:
        s = np.logspace(0, -4, 72)   # every value resolved by the Gram route
    x, M = _dense_ac2(rng, Dl, Dr, s)
    atol = 1e-10
    ctx.set_svd_method("gram")
    try:
        al, S, ar, eps = mpsgb.svd_trunc(mpsgb.DeviceTensor.from_numpy(ctx, "ac2", x), None, atol,
                                         normalize=False)
    finally:
        ctx.set_svd_method("gesvd")
    Uo, So, Vo, eo = P.svd_trunc(M, None, atol)
    assert al.dims[2] == So.size
    assert abs(eps - eo) <= 1e-12 + 1e-6 * eo
    # the same truncated matrix
    dev = np.einsum("lsk,km,mtr->lsrt", al.numpy(), S.numpy(), ar.numpy())
    ref = ((Uo * So) @ Vo).reshape(Dl, 2, 2, Dr, order="F").transpose(0, 1, 3, 2)
    assert np.abs(dev - ref).max() < 1e-10
    # deep spectra took the SVD (diagonal S), benign ones stayed on the Gram route
    # (triangular S = R Sigma)
    assert _is_diag(S.numpy()) == (spread == "deep")


def test_u1_gram_truncation_matches_svd(ctx):
    rng = np.random.default_rng(12)
    ql = np.sort(rng.integers(-2, 3, size=30)).astype(np.int32)
    qr = np.sort(rng.integers(-2, 3, size=34)).astype(np.int32)
    m, n = 2 * len(ql), 2 * len(qr)
    qrow = (ql[:, None] + QP[None, :]).reshape(-1, order="F")   # rows (l, s1)
    qcol = (qr[:, None] - QP[None, :]).reshape(-1, order="F")   # columns (r, s2)
    M = np.zeros((m, n))
    for q in np.intersect1d(qrow, qcol):
        r, c = np.flatnonzero(qrow == q), np.flatnonzero(qcol == q)
        k = min(r.size, c.size)
        s = np.logspace(-0.3 * abs(q), -12 - 0.3 * abs(q), k)  # each block spans 12 decades
        M[np.ix_(r, c)] = _orth(rng, r.size, k) @ np.diag(s) @ _orth(rng, c.size, k).T
    AC2 = M.reshape(len(ql), 2, len(qr), 2, order="F")
    atol = 1e-10
    t = mpsgb.DeviceTensor.from_numpy(ctx, "ac2", AC2)
    t.charges = (ql, QP, qr, QP)
    ctx.set_svd_method("gram")
    try:
        al, S, ar, eps = mpsgb.svd_trunc(t, None, atol, normalize=False)
    finally:
        ctx.set_svd_method("gesvd")
    Uu, Sv, Vh, qk, oeps = U.svd_trunc_u1(M, qrow, qcol, None, atol)
    assert np.array_equal(al.charges[2], qk)
    assert abs(eps - oeps) <= 1e-12 + 1e-6 * oeps
    dev = np.einsum("lsk,km,mtr->lsrt", al.numpy(), S.numpy(), ar.numpy())
    ref = ((Uu * Sv) @ Vh).reshape(AC2.shape, order="F")
    assert np.abs(dev - ref).max() < 1e-10
    assert np.all(al.numpy()[~HU.block_mask(ql, QP, qk)] == 0)
