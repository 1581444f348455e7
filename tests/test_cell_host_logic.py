"""Host logic of the unit-cell drivers (mpsgb/cell.py) on the CPU: every device operation the
drivers call is replaced by a numpy stand-in with the same meaning (module globals patched for
the test), and the orchestration -- cell gauge fixing, level-by-level cell environments, VUMPS
and IDMRG2 -- is run against the oracle's independent restatement (oracle/cell.py).  The device
operations themselves are covered by the GPU tests."""
import numpy as np
import pytest

import mpsgb
from oracle import cell as Ce
from oracle import derivatives as dv
from oracle import models as M
from oracle.krylov import lanczos_eigsolve
from oracle.mps import lq_pos, qr_pos, svd_trunc as np_svd


class Ctx:
    handle = None


CTX = Ctx()


class T:
    """Stand-in for DeviceTensor: a numpy array in the reference leg order."""

    def __init__(self, ctx, kind, dtype, dims, handle=None, charges=None):
        self.ctx, self.kind = ctx, kind
        self.a = np.zeros(dims, dtype=dtype)
        self.charges = None

    @property
    def handle(self):
        return self

    @property
    def dims(self):
        return tuple(self.a.shape)

    @property
    def dtype(self):
        return self.a.dtype

    @staticmethod
    def from_numpy(ctx, kind, arr, dtype=None):
        t = T(ctx, kind, np.dtype(dtype or np.asarray(arr).dtype), np.shape(arr))
        t.a = np.array(arr, dtype=t.a.dtype)
        return t

    @staticmethod
    def of(a):
        t = T(CTX, 0, a.dtype, a.shape)
        t.a = np.array(a)
        return t

    def copy(self):
        return T.of(self.a)

    def scale_(self, s):
        if s == 0:
            self.a = np.zeros_like(self.a)
        else:
            self.a = self.a * (s if self.a.dtype.kind == "c" else np.real(s))
        return self

    def axpy_(self, s, x):
        self.a = self.a + (s if self.a.dtype.kind == "c" else np.real(s)) * x.a
        return self

    def dot(self, o):
        v = np.vdot(self.a, o.a)
        return v if self.a.dtype.kind == "c" else float(np.real(v))

    def norm(self):
        return float(np.linalg.norm(self.a))

    def normalize_(self):
        return self.scale_(1.0 / self.norm())

    def numpy(self):
        return np.array(self.a)


def left_orth(AC):
    Dl, d, Dr = AC.dims
    Q, R = qr_pos(AC.a.reshape(Dl * d, Dr, order="F"))
    return T.of(Q.reshape(Dl, d, Q.shape[1], order="F")), T.of(R)


def right_orth(AC):
    Dl, d, Dr = AC.dims
    Lm, Q = lq_pos(AC.a.reshape(Dl, d * Dr, order="F"))
    return T.of(Lm), T.of(Q.reshape(Q.shape[0], d, Dr, order="F"))


def mul_front(C, A):
    return T.of(np.einsum("ab,bsc->asc", C.a, A.a))


def mul_tail(A, C):
    return T.of(np.einsum("asb,bc->asc", A.a, C.a))


def ac2_from(A, B):
    return T.of(np.einsum("asm,mtb->asbt", A.a, B.a))


def svd_trunc(x, maxdim=None, atol=0.0, normalize=True):
    Dl, d1, Dr, d2 = x.dims
    U, S, Vh, eps = np_svd(x.a.reshape(Dl * d1, Dr * d2, order="F"), maxdim, atol)
    if normalize:
        S = S / np.linalg.norm(S)
    k = S.size
    al = U.reshape(Dl, d1, k, order="F")
    ar = np.transpose(Vh.reshape(k, Dr, d2, order="F"), (0, 2, 1))
    return T.of(al), T.of(np.diag(S).astype(x.a.dtype)), T.of(ar), eps


def _transfer(side, ctx, env, Wb, A, prec):
    if side == "L":
        return T.of(dv.transfer_left(env.a, Wb.a, A.a, A.a))
    return T.of(dv.transfer_right(env.a, Wb.a, A.a, A.a))


def _regularize(ctx, x, lvec, rvec):
    lam = np.einsum("xy,ywx->w", lvec.a, x.a)
    x.a = x.a - lam[None, :, None] * rvec.a[:, None, :]
    return x


def _transfer_bond(side, A, B, X):
    if side == 0:
        return T.of(np.einsum("lsb,lm,msa->ba", B.a.conj(), X.a, A.a))
    return T.of(np.einsum("asr,rq,bsq->ab", A.a, X.a, B.a.conj()))


def _as_mps(C):
    return T.of(C.a.reshape(C.a.shape[0], 1, C.a.shape[1]))


def _as_bond(A):
    return T.of(A.a.reshape(A.a.shape[0], A.a.shape[2]))


def _adj(C):
    return T.of(C.a.conj().T)


def _diff_norm(a, b):
    return float(np.linalg.norm(a.a - b.a))


def _arnoldi_dominant(op, x0, tol, krylovdim=30, maxiter=200):
    D0, D1 = x0.dims
    n = D0 * D1
    M_ = np.zeros((n, n), dtype=np.complex128)
    for k in range(n):
        e = np.zeros(n, dtype=np.complex128)
        e[k] = 1
        M_[:, k] = op(T.of(e.reshape(D0, D1, order="F").astype(x0.a.dtype))).a.reshape(-1, order="F")
    ev, U = np.linalg.eig(M_)
    v = U[:, np.argmax(np.abs(ev))].reshape(D0, D1, order="F")
    if x0.a.dtype.kind != "c":
        v = v.real
    return T.of(v / np.linalg.norm(v))


def regauge(AC, C):
    return T.of(Ce._regauge(AC.a, C.a))


def project_complement_(y, AL):
    D, d, Dr = AL.dims
    A = AL.a.reshape(D * d, Dr, order="F")
    Y = y.a.reshape(D * d, -1, order="F")
    y.a = (Y - A @ (A.conj().T @ Y)).reshape(y.a.shape, order="F")
    return y


class Op:
    """Stand-in for DerivativeOperator: the oracle's prepared C / AC / AC2 maps."""

    def __init__(self, ctx, kind, GL, W1, W2, GR, backend):
        self.kind, self.GL, self.W1, self.W2, self.GR = kind, GL.a, W1, W2, GR.a

    def __call__(self, x):
        if self.kind == mpsgb._lib.GB_HEFF_C:
            return T.of(dv.CHam(self.GL, self.GR)(x.a))
        if self.kind == mpsgb._lib.GB_HEFF_AC:
            if self.W1.a.shape[3] == 1:
                return T.of(dv.mpo_ac_apply(self.GL, self.W1.a, self.GR, x.a))
            return T.of(dv.JordanAC(self.GL, self.W1.a, self.GR)(x.a))
        return T.of(dv.JordanAC2(self.GL, self.W1.a, self.W2.a, self.GR)(x.a))


def fixedpoint(op, x0, which, solver):
    val, vec, info = lanczos_eigsolve(op_np(op), x0.a, krylovdim=solver.krylovdim,
                                      maxiter=solver.maxiter, tol=solver.tol, eager=solver.eager)
    return val, T.of(vec), info


def op_np(op):
    return lambda x: op(T.of(x)).a


class FakeLib:
    def gb_env_channel_copy(self, ctx, dst, doff, src, soff, n):
        dst.a[:, doff:doff + n, :] = src.a[:, soff:soff + n, :]
        return 0


class FakeL:
    GB_KIND_MPS = mpsgb._lib.GB_KIND_MPS
    GB_KIND_BOND = mpsgb._lib.GB_KIND_BOND
    GB_KIND_GL = mpsgb._lib.GB_KIND_GL
    GB_KIND_GR = mpsgb._lib.GB_KIND_GR
    GB_KIND_MPO = mpsgb._lib.GB_KIND_MPO
    GB_KIND_AC2 = mpsgb._lib.GB_KIND_AC2
    GB_HEFF_AC = mpsgb._lib.GB_HEFF_AC
    GB_HEFF_C = mpsgb._lib.GB_HEFF_C
    GB_HEFF_AC2 = mpsgb._lib.GB_HEFF_AC2
    GB_PREC_FP64 = mpsgb._lib.GB_PREC_FP64

    @staticmethod
    def lib():
        return FakeLib()

    @staticmethod
    def check(rc):
        return rc


class Hdev:
    """The product's MPOHamiltonian with stand-in device copies of its tensors."""

    def __init__(self, H):
        self.H = H
        self.W = H.W
        self.chans = H.chans
        self.dtype = H.dtype

    def __len__(self):
        return len(self.H)

    def device(self, ctx, dtype=None):
        return [T.of(w.astype(dtype or w.dtype)) for w in self.W]


@pytest.fixture
def GC(monkeypatch):
    """mpsgb.cell with its device operations replaced by the numpy stand-ins above."""
    import mpsgb.cell as cell
    stand_ins = dict(DeviceTensor=T, left_orth=left_orth, right_orth=right_orth,
                     mul_front=mul_front, mul_tail=mul_tail, ac2_from=ac2_from,
                     svd_trunc=svd_trunc, _transfer=_transfer, _regularize=_regularize,
                     _transfer_bond=_transfer_bond, _as_mps=_as_mps, _adj=_adj,
                     _as_bond_t=_as_bond, _diff_norm=_diff_norm,
                     _arnoldi_dominant=_arnoldi_dominant, regauge=regauge,
                     project_complement_=project_complement_, DerivativeOperator=Op,
                     fixedpoint=fixedpoint, L=FakeL, context=lambda *a: CTX,
                     _inv_bond=lambda C: T.of(np.linalg.inv(C.a)))
    for name, f in stand_ins.items():
        monkeypatch.setattr(cell, name, f)
    return cell




def _tfim2(g=0.5):
    H = mpsgb.transverse_field_ising(2, g=g, infinite=True)
    oH = M.infinite_mpo_hamiltonian(2, 2, M.tfim_terms(2, g=g, periodic=True))
    return Hdev(H), oH


def _As(D, seed):
    rng = np.random.default_rng(seed)
    return [rng.standard_normal((D, 2, D)) + 1j * rng.standard_normal((D, 2, D))
            for _ in range(2)]


def test_cell_gauge_and_environments(GC):
    Hd, oH = _tfim2()
    As = _As(10, 21)
    opsi = Ce.infinite_mps(As)
    psi = GC.InfiniteMPSCell.from_tensors(As, CTX)
    AL, AR, C = psi.to_numpy()
    for s in range(2):
        assert np.allclose(AL[s], opsi.AL[s], atol=1e-12)
        assert np.allclose(AR[s], opsi.AR[s], atol=1e-12)
        assert np.allclose(C[s], opsi.C[s], atol=1e-12)
    envs = GC.InfiniteEnvironmentsCell(psi, Hd).recalculate(psi, tol=1e-12)
    GL, GR = Ce.infinite_envs(opsi, oH, tol=1e-12)
    for s in range(2):
        assert np.allclose(envs.GL[s].a, GL[s], atol=1e-10)
        assert np.allclose(envs.GR[s].a, GR[s], atol=1e-10)
    assert abs(GC.energy(psi, envs) - Ce.energy(opsi, oH, GL, GR)) < 1e-12


def test_cell_vumps_orchestration(GC):
    Hd, oH = _tfim2()
    As = _As(10, 21)
    _, _, _, oeps, ohist = Ce.vumps(Ce.infinite_mps(As), oH, tol=1e-10, maxiter=50)
    psi = GC.InfiniteMPSCell.from_tensors(As, CTX)
    _, _, eps, hist = GC.find_groundstate_vumps(psi, Hd, mpsgb.VUMPS(tol=1e-10, maxiter=50))
    assert len(hist) == len(ohist)
    assert eps <= 1e-10
    assert abs(hist[-1]["energy"] - ohist[-1][1]) < 1e-12


def test_idmrg2_orchestration(GC):
    Hd, oH = _tfim2()
    As = _As(4, 22)
    opsi, oGL, oGR, oeps, ohist = Ce.idmrg2(Ce.infinite_mps(As), oH, maxdim=16, atol=1e-10,
                                            tol=1e-10, maxiter=50)
    psi = GC.InfiniteMPSCell.from_tensors(As, CTX)
    psi, envs, eps, hist = GC.find_groundstate_idmrg2(
        psi, Hd, GC.IDMRG2(maxdim=16, cutoff=1e-10, tol=1e-10, maxiter=50))
    assert len(hist) == len(ohist)
    assert abs(GC.energy(psi, envs) - Ce.energy(opsi, oH, oGL, oGR)) < 1e-12
    assert abs(hist[-1]["energy_change"] - ohist[-1][1]) < 1e-10


def test_infinite_drivers_hand_cells_to_the_cell_forms(monkeypatch):
    """find_groundstate_vumps / find_groundstate_idmrg / timestep_infinite take an
    InfiniteMPSCell to the cell forms (one entry point per algorithm, as the reference's
    find_groundstate and timestep take any unit cell)."""
    import mpsgb
    from mpsgb import cell, infinite
    seen = []
    monkeypatch.setattr(cell, "find_groundstate_vumps", lambda *a: seen.append("vumps") or a)
    monkeypatch.setattr(cell, "find_groundstate_idmrg", lambda *a: seen.append("idmrg") or a)
    monkeypatch.setattr(cell, "timestep", lambda *a: seen.append("tdvp") or a)
    psi = cell.InfiniteMPSCell([], [], [])
    infinite.find_groundstate_vumps(psi, None, None)
    infinite.find_groundstate_idmrg(psi, None, None)
    out = infinite.timestep_infinite(psi, None, 0.0, 0.1, None, None, True, 1e-12)
    assert seen == ["vumps", "idmrg", "tdvp"]
    assert out == (psi, None, 0.0, 0.1, None, None, True, 1e-12)
    assert mpsgb.InfiniteMPSCell is cell.InfiniteMPSCell and mpsgb.IDMRG2 is cell.IDMRG2
