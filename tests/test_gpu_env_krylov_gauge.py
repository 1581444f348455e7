"""GPU parity of environment transfers, Krylov solvers and gauge factorisations."""
import numpy as np
import pytest
import scipy.linalg as sl

import mpsgb
from mpsgb import _lib as L
from oracle import derivatives as dv
from oracle import krylov as K
from oracle import models as M
from oracle import mps as P

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    return mpsgb.context(0)


def _rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.mark.parametrize("dt", [np.float64, np.complex128])
@pytest.mark.parametrize("prec,tol", [("fp64", 1e-12), ("bf16x3", 1e-4), ("tf32x3", 4e-6)])
def test_transfers(ctx, dt, prec, tol):
    L_ = 10
    H = M.finite_mpo_hamiltonian(L_, 2, M.j1j2_cylinder_terms(5, 2) if dt == np.float64
                                 else M.heisenberg_terms(L_), dtype=dt)
    psi = P.finite_mps_from_tensors(P.random_initial_tensors(L_, 2, 24, 31, dt))
    envs = P.FiniteEnvironments(psi, H)
    code = L.PRECISIONS[prec]
    for j in (0, 3, 7):
        GL = envs.leftenv(j, psi)
        A = psi.AL[j]
        ref = dv.transfer_left(GL, H[j], A, A)
        g = mpsgb.DeviceTensor.from_numpy(ctx, "gl", GL)
        w = mpsgb.DeviceTensor.from_numpy(ctx, "mpo", H[j])
        a = mpsgb.DeviceTensor.from_numpy(ctx, "mps", A)
        out = mpsgb.DeviceTensor(ctx, "gl", dt, ref.shape)
        L.check(L.lib().gb_env_transfer_left(ctx.handle, g.handle, w.handle, a.handle, a.handle,
                                             code, out.handle))
        assert _rel(out.numpy(), ref) < tol
        GR = envs.rightenv(j, psi)
        B = psi.AR[j]
        ref = dv.transfer_right(GR, H[j], B, B)
        r = mpsgb.DeviceTensor.from_numpy(ctx, "gr", GR)
        b = mpsgb.DeviceTensor.from_numpy(ctx, "mps", B)
        out = mpsgb.DeviceTensor(ctx, "gr", dt, ref.shape)
        L.check(L.lib().gb_env_transfer_right(ctx.handle, r.handle, w.handle, b.handle, b.handle,
                                              code, out.handle))
        assert _rel(out.numpy(), ref) < tol


def test_eigsolve_matches_oracle_and_dense(ctx):
    L_ = 8
    H = M.finite_mpo_hamiltonian(L_, 2, M.xxz_terms(L_, 1.0, 1.3, 0.1))
    psi = P.finite_mps_from_tensors(P.random_initial_tensors(L_, 2, 8, 41))
    envs = P.FiniteEnvironments(psi, H)
    pos = 3
    GL, GR = envs.leftenv(pos, psi), envs.rightenv(pos + 1, psi)
    op_ref = dv.JordanAC2(GL, H[pos], H[pos + 1], GR)
    rng = np.random.default_rng(3)
    x = rng.standard_normal((GL.shape[0], 2, GR.shape[0], 2)) + 0j
    g = mpsgb.DeviceTensor.from_numpy(ctx, "gl", GL)
    r = mpsgb.DeviceTensor.from_numpy(ctx, "gr", GR)
    w1 = mpsgb.DeviceTensor.from_numpy(ctx, "mpo", H[pos])
    w2 = mpsgb.DeviceTensor.from_numpy(ctx, "mpo", H[pos + 1])
    op = mpsgb.DerivativeOperator(ctx, L.GB_HEFF_AC2, g, w1, w2, r, mpsgb.GB300Backend())
    n = x.size
    Hd = np.zeros((n, n), dtype=np.complex128)
    for i in range(n):
        e = np.zeros(n, dtype=np.complex128)
        e[i] = 1
        Hd[:, i] = op_ref(e.reshape(x.shape, order="F")).ravel(order="F")
    exact = np.linalg.eigvalsh(Hd)[0]
    for kd, mi in ((30, 50), (8, 100)):   # the second one exercises thick restarts
        val, vec, info = mpsgb.fixedpoint(op, mpsgb.DeviceTensor.from_numpy(ctx, "ac2", x), "SR",
                                          mpsgb.Lanczos(kd, mi, 1e-11, False))
        oval, ovec, oinfo = K.lanczos_eigsolve(op_ref, x, krylovdim=kd, maxiter=mi, tol=1e-11)
        assert abs(val - exact) < 1e-9
        assert abs(val - oval) < 1e-10
        assert info.converged >= 1
        v = vec.numpy()
        assert abs(abs(np.vdot(v, ovec)) - 1) < 1e-8
        # residual of the returned Ritz pair
        res = op_ref(v) - val * v
        assert np.linalg.norm(res) < 1e-9


def test_eigsolve_adaptive_budget_counts(ctx):
    """krylovdim=3, maxiter=1 (the AdaptiveKrylov cold start) uses exactly 3 matvecs."""
    L_ = 8
    H = M.finite_mpo_hamiltonian(L_, 2, M.heisenberg_terms(L_))
    psi = P.finite_mps_from_tensors(P.random_initial_tensors(L_, 2, 8, 42))
    envs = P.FiniteEnvironments(psi, H)
    pos = 2
    GL, GR = envs.leftenv(pos, psi), envs.rightenv(pos + 1, psi)
    op_ref = dv.JordanAC2(GL, H[pos], H[pos + 1], GR)
    op = mpsgb.DerivativeOperator(ctx, L.GB_HEFF_AC2, mpsgb.DeviceTensor.from_numpy(ctx, "gl", GL),
                                  mpsgb.DeviceTensor.from_numpy(ctx, "mpo", H[pos]),
                                  mpsgb.DeviceTensor.from_numpy(ctx, "mpo", H[pos + 1]),
                                  mpsgb.DeviceTensor.from_numpy(ctx, "gr", GR), mpsgb.GB300Backend())
    x = np.random.default_rng(4).standard_normal((GL.shape[0], 2, GR.shape[0], 2)) + 0j
    val, vec, info = mpsgb.fixedpoint(op, mpsgb.DeviceTensor.from_numpy(ctx, "ac2", x), "SR",
                                      mpsgb.Lanczos(3, 1, 1e-12, True))
    oval, _, oinfo = K.lanczos_eigsolve(op_ref, x, krylovdim=3, maxiter=1, tol=1e-12, eager=True)
    assert info.numops == oinfo.numops == 3
    assert abs(val - oval) < 1e-11
    assert abs(info.normres - oinfo.normres) < 1e-9


def test_exponentiate_matches_expm(ctx):
    L_ = 6
    H = M.finite_mpo_hamiltonian(L_, 2, M.heisenberg_terms(L_))
    psi = P.finite_mps_from_tensors(P.random_initial_tensors(L_, 2, 4, 43))
    envs = P.FiniteEnvironments(psi, H)
    pos = 2
    GL, GR = envs.leftenv(pos, psi), envs.rightenv(pos, psi)
    op_ref = dv.JordanAC(GL, H[pos], GR)
    op = mpsgb.DerivativeOperator(ctx, L.GB_HEFF_AC, mpsgb.DeviceTensor.from_numpy(ctx, "gl", GL),
                                  mpsgb.DeviceTensor.from_numpy(ctx, "mpo", H[pos]), None,
                                  mpsgb.DeviceTensor.from_numpy(ctx, "gr", GR), mpsgb.GB300Backend())
    x = np.random.default_rng(5).standard_normal((GL.shape[0], 2, GR.shape[0])) + 0j
    n = x.size
    Hd = np.zeros((n, n), dtype=np.complex128)
    for i in range(n):
        e = np.zeros(n, dtype=np.complex128)
        e[i] = 1
        Hd[:, i] = op_ref(e.reshape(x.shape, order="F")).ravel(order="F")
    for t in (-0.3j, -0.05, -1.5j):
        y, info = mpsgb.exponentiate(op, t, mpsgb.DeviceTensor.from_numpy(ctx, "mps", x),
                                     mpsgb.Lanczos(20, 100, 1e-12))
        ref = (sl.expm(t * Hd) @ x.ravel(order="F")).reshape(x.shape, order="F")
        assert _rel(y.numpy(), ref) < 1e-10
        assert info.converged == 1


@pytest.mark.parametrize("dt", [np.float64, np.complex128])
@pytest.mark.parametrize("shape", [(6, 2, 5, 2), (3, 2, 9, 2), (8, 2, 8, 2)])
def test_svd_trunc(ctx, dt, shape):
    rng = np.random.default_rng(6)
    x = rng.standard_normal(shape)
    if np.dtype(dt).kind == "c":
        x = x + 1j * rng.standard_normal(shape)
    x = x.astype(dt)
    Dl, d1, Dr, d2 = shape
    M_ = x.reshape(Dl * d1, Dr * d2, order="F")
    for maxdim in (4, 100):
        al, S, ar, eps = mpsgb.svd_trunc(mpsgb.DeviceTensor.from_numpy(ctx, "ac2", x), maxdim, 0.0,
                                         normalize=False)
        U, s, Vh, e = P.svd_trunc(M_, maxdim, 0.0)
        k = s.size
        assert al.dims == (Dl, d1, k) and ar.dims == (k, d2, Dr)
        assert np.allclose(np.diag(S.numpy()).real, s, atol=1e-12)
        assert abs(eps - e) < 1e-10
        # reconstruction of the rank-k approximation
        rec = np.einsum("asm,mn,ntb->asbt", al.numpy(), S.numpy(), ar.numpy())
        ref = (U * s) @ Vh
        assert np.allclose(rec.reshape(Dl * d1, Dr * d2, order="F"), ref, atol=1e-11)
        A = al.numpy().reshape(Dl * d1, k, order="F")
        assert np.allclose(A.conj().T @ A, np.eye(k), atol=1e-12)


@pytest.mark.parametrize("dt", [np.float64, np.complex128])
@pytest.mark.parametrize("shape", [(4, 2, 8), (8, 2, 5), (5, 2, 5)])
def test_left_right_orth(ctx, dt, shape):
    rng = np.random.default_rng(7)
    a = rng.standard_normal(shape)
    if np.dtype(dt).kind == "c":
        a = a + 1j * rng.standard_normal(shape)
    a = a.astype(dt)
    Dl, d, Dr = shape
    q, r = mpsgb.left_orth(mpsgb.DeviceTensor.from_numpy(ctx, "mps", a))
    Q, R = P.qr_pos(a.reshape(Dl * d, Dr, order="F"))
    assert np.allclose(q.numpy().reshape(Dl * d, -1, order="F"), Q, atol=1e-12)
    assert np.allclose(r.numpy(), R, atol=1e-12)
    l, q2 = mpsgb.right_orth(mpsgb.DeviceTensor.from_numpy(ctx, "mps", a))
    Lm, Q2 = P.lq_pos(a.reshape(Dl, d * Dr, order="F"))
    assert np.allclose(l.numpy(), Lm, atol=1e-12)
    assert np.allclose(q2.numpy().reshape(q2.dims[0], -1, order="F"), Q2, atol=1e-12)


@pytest.mark.parametrize("dt", [np.float64, np.complex128])
@pytest.mark.parametrize("shape", [(6, 2, 5, 2), (3, 2, 9, 2), (8, 2, 8, 2)])
@pytest.mark.parametrize("method", ["gesvdp", "gram"])
def test_svd_trunc_methods(ctx, dt, shape, method):
    """The alternative factorisations give the same truncated state with exactly
    isometric AL and AR (the Gram method returns a triangular bond matrix)."""
    rng = np.random.default_rng(8)
    x = rng.standard_normal(shape)
    if np.dtype(dt).kind == "c":
        x = x + 1j * rng.standard_normal(shape)
    x = x.astype(dt)
    Dl, d1, Dr, d2 = shape
    M_ = x.reshape(Dl * d1, Dr * d2, order="F")
    ctx.set_svd_method(method)
    try:
        for maxdim in (4, 100):
            al, C, ar, eps = mpsgb.svd_trunc(mpsgb.DeviceTensor.from_numpy(ctx, "ac2", x), maxdim,
                                             0.0, normalize=False)
            U, s, Vh, e = P.svd_trunc(M_, maxdim, 0.0)
            k = s.size
            assert abs(eps - e) < 1e-9
            rec = np.einsum("asm,mn,ntb->asbt", al.numpy(), C.numpy(), ar.numpy())
            ref = (U * s) @ Vh
            assert np.allclose(rec.reshape(Dl * d1, Dr * d2, order="F"), ref, atol=1e-10)
            A = al.numpy().reshape(Dl * d1, k, order="F")
            B = ar.numpy().reshape(k, d2 * Dr, order="F")
            assert np.allclose(A.conj().T @ A, np.eye(k), atol=1e-12)
            assert np.allclose(B @ B.conj().T, np.eye(k), atol=1e-12)
    finally:
        ctx.set_svd_method("gesvd")
