"""U(1) symmetry on the CPU: the oracle's block-wise factorisations, the symmetric random
states and MPO channels of the host package, and U(1) DMRG2 against exact diagonalisation
in the Sz = 0 sector."""
import numpy as np
import pytest

from oracle import models as M
from oracle import mps as P
from oracle import u1 as U

from mpsgb import operators as O
from mpsgb import u1 as HU


def _sym_matrix(rng, qrow, qcol, dtype=np.float64):
    A = rng.standard_normal((len(qrow), len(qcol)))
    if np.dtype(dtype).kind == "c":
        A = A + 1j * rng.standard_normal(A.shape)
    return (A * (np.asarray(qrow)[:, None] == np.asarray(qcol)[None, :])).astype(dtype)


@pytest.mark.parametrize("dtype", [np.float64, np.complex128])
def test_left_right_orth_u1_invariants(dtype):
    rng = np.random.default_rng(3)
    qrow = np.sort(rng.integers(-3, 4, size=40))
    qcol = np.sort(rng.integers(-3, 4, size=25))
    A = _sym_matrix(rng, qrow, qcol, dtype)
    Q, R, qk = U.left_orth_u1(A, qrow, qcol)
    assert np.allclose(Q @ R, A, atol=1e-13)
    assert np.allclose(Q.conj().T @ Q, np.eye(Q.shape[1]), atol=1e-13)
    # structure: Q only couples equal charges, and exactly so
    assert np.all(Q[np.asarray(qrow)[:, None] != qk[None, :]] == 0)
    assert np.all(np.diff(qk) >= 0)
    Lm, Q2, qk2 = U.right_orth_u1(A, qrow, qcol)
    assert np.allclose(Lm @ Q2, A, atol=1e-13)
    assert np.allclose(Q2 @ Q2.conj().T, np.eye(Q2.shape[0]), atol=1e-13)
    assert np.all(Q2[qk2[:, None] != np.asarray(qcol)[None, :]] == 0)


def test_svd_trunc_u1_spectrum_and_truncation():
    rng = np.random.default_rng(5)
    qrow = np.sort(rng.integers(-2, 3, size=30))
    qcol = np.sort(rng.integers(-2, 3, size=30))
    A = _sym_matrix(rng, qrow, qcol)
    Uu, S, Vh, qk, eps = U.svd_trunc_u1(A, qrow, qcol)
    assert np.allclose((Uu * S) @ Vh, A, atol=1e-12)
    assert np.allclose(np.sort(S), np.sort(np.linalg.svd(A, compute_uv=False)[:S.size]),
                       atol=1e-12)
    assert eps < 1e-12
    Uk, Sk, Vk, qkk, epsk = U.svd_trunc_u1(A, qrow, qcol, maxdim=7)
    full = np.sort(np.linalg.svd(A, compute_uv=False))[::-1]
    assert np.allclose(np.sort(Sk)[::-1], full[:7], atol=1e-12)
    assert abs(epsk - np.linalg.norm(full[7:])) < 1e-12


def test_bond_charges_and_random_states():
    qb = HU.bond_charges(24, 64, 0)
    assert len(qb) == 25 and qb[0].tolist() == [0] and qb[-1].tolist() == [0]
    assert max(len(q) for q in qb) <= 64
    for q in qb:
        assert np.all(np.diff(q) >= 0)
    As, qb = HU.random_u1_tensors(12, 16, 7, 0, np.float64)
    for i, a in enumerate(As):
        mask = HU.block_mask(qb[i], O.SPIN_HALF_CHARGES, qb[i + 1])
        assert np.all(a[~mask] == 0) and np.any(a[mask] != 0)


def test_u1_mpo_equals_plain_mpo():
    """Charge-definite channels give the same operator (dense contraction, L = 6)."""
    def full(H):
        res = H.W[0]
        for w in H.W[1:]:
            res = np.einsum("aijb,bklc->aikjlc", res, w)
            s = res.shape
            res = res.reshape(s[0], s[1] * s[2], s[3] * s[4], s[5])
        return res[0, :, :, -1]
    a = full(O.heisenberg_XXX(6, dtype=np.float64))
    b = full(O.heisenberg_XXX(6, dtype=np.float64, u1=True))
    assert np.abs(a - b).max() < 1e-14
    # every channel of the U(1) MPO carries one charge: W[a, s, t, b] != 0 only for
    # q_in(a) + q(s) = q(t) + q_out(b) with a consistent channel charge assignment
    W = O.heisenberg_XXX(6, dtype=np.float64, u1=True).W[2]
    q = O.SPIN_HALF_CHARGES
    for b in range(W.shape[3]):
        nz = np.argwhere(np.abs(W[:, :, :, b]) > 0)
        deltas = {int(q[s] - q[t]) for (a, s, t) in nz if a == 0}
        assert len(deltas) <= 1


def test_u1_dmrg2_matches_ed_sector():
    L_, D = 10, 24
    As, qb = HU.random_u1_tensors(L_, D, 11, 0, np.float64)
    H = O.heisenberg_XXX(L_, dtype=np.float64, u1=True)
    psi = P.finite_mps_from_tensors(As, charges=(qb, O.SPIN_HALF_CHARGES))
    psi, envs, eps, hist = P.find_groundstate_dmrg2(psi, H, P.DMRG2(maxdim=D, cutoff=1e-12),
                                                    maxsweeps=8)
    e_ed = M.ed_ground_energy(L_, 2, M.heisenberg_terms(L_, dtype=np.float64))[0]
    assert abs(hist[-1][1] - e_ed) < 1e-7 * abs(e_ed)
    # the state stayed block sparse with charge-sorted bonds
    for i in range(L_ - 1):
        a = psi.AL[i] if psi.AL[i] is not None and i < psi.center else None
        if a is not None:
            mask = HU.block_mask(psi.qb[i], psi.qp, psi.qb[i + 1])
            assert np.all(a[~mask] == 0)


def test_mpo_channel_charges_host_and_oracle_agree():
    """The charge labels of the MPO channels: every nonzero W[a, s, t, c] moves q_s - q_t into
    the channel, for plain, summed and product Hamiltonians."""
    L_ = 6
    H = O.heisenberg_XXX(L_, dtype=np.float64, u1=True)
    cyl = O.j1j2_cylinder(4, 6, dtype=np.float64, u1=True)     # long-range channels
    for Hx in (H, H + O.xxz(L_, 0.0, 1.0, 0.2, dtype=np.float64, u1=True), H * H, cyl):
        qh = HU.channel_charges(Hx.W, O.SPIN_HALF_CHARGES)
        qo = U.mpo_channel_charges(Hx.W, O.SPIN_HALF_CHARGES)
        qp = np.asarray(O.SPIN_HALF_CHARGES)
        for i, w in enumerate(Hx.W):
            assert np.array_equal(qh[i], qo[i])
            for a, s, t, c in np.argwhere(w != 0):
                assert qh[i + 1][c] == qh[i][a] + qp[s] - qp[t]
        assert qh[0].tolist() == [0] and qh[-1].tolist() == [0]
    with pytest.raises(ValueError):
        HU.channel_charges(O.heisenberg_XXX(L_, dtype=np.float64).W, O.SPIN_HALF_CHARGES)


@pytest.mark.parametrize("right", [True, False])
def test_u1_dmrg3s_perturbation_is_block_sparse(right):
    """The DMRG3S perturbation of a U(1) state lives on the charge blocks of the fused
    (bond, channel) leg, so the enlarged tensor is symmetric and its bond sorts by charge."""
    L_, pos = 8, 3
    H = O.heisenberg_XXX(L_, dtype=np.float64, u1=True)
    As, qb = HU.random_u1_tensors(L_, 8, 4, 0, np.float64)
    psi = P.finite_mps_from_tensors(As, charges=(qb, O.SPIN_HALF_CHARGES))
    psi.center = pos if right else pos + 1          # every AL, AR and C is valid
    envs = P.FiniteEnvironments(psi, H)
    AC = psi.ac(pos)
    v0 = [psi.qb[b].copy() for b in range(L_ + 1)]
    P.dmrg3s_gauge(pos, right, psi, H, envs, AC, 0.3, 64, 0.0)
    b = pos + 1 if right else pos
    qk = psi.qb[b]
    assert np.all(np.diff(qk) >= 0) and len(qk) > len(v0[b])
    if right:
        A, ql, qr = psi.AL[pos], psi.qb[pos], qk
    else:
        A, ql, qr = psi.AR[pos], qk, psi.qb[pos + 1]
    mask = HU.block_mask(ql, psi.qp, qr)
    assert np.all(A[~mask] == 0)
    m = A.reshape(-1, A.shape[2], order="F") if right else A.reshape(A.shape[0], -1, order="F")
    g = m.conj().T @ m if right else m @ m.conj().T
    assert np.abs(g - np.eye(len(g))).max() < 1e-12


def test_u1_single_site_dmrg3s_reaches_ed():
    L_ = 10
    As, qb = HU.random_u1_tensors(L_, 2, 5, 0, np.float64)
    H = O.heisenberg_XXX(L_, dtype=np.float64, u1=True)
    psi = P.finite_mps_from_tensors(As, charges=(qb, O.SPIN_HALF_CHARGES))
    alg = P.DMRG(tol=1e-10, maxiter=12, alg_gauge=P.DMRG3S(0.1, 0.8, 16, 1e-12))
    psi, envs, eps, hist = P.find_groundstate_dmrg(psi, H, alg)
    e_ed = M.ed_ground_energy(L_, 2, M.heisenberg_terms(L_, dtype=np.float64))[0]
    assert -1e-12 * abs(e_ed) <= hist[-1][1] - e_ed < 1e-7 * abs(e_ed), (hist[-1], e_ed)


def _dense_state(psi):
    """The state vector of an oracle FiniteMPS (AL left of the centre bond, AR right of it)."""
    T = np.ones((1, 1))
    for i in range(psi.center):
        T = np.tensordot(T, psi.AL[i], axes=([-1], [0]))
    T = np.tensordot(T, psi.C[psi.center], axes=([-1], [0]))
    for i in range(psi.center, len(psi)):
        T = np.tensordot(T, psi.AR[i], axes=([-1], [0]))
    return T.reshape(-1)


@pytest.mark.parametrize("right", [True, False])
@pytest.mark.parametrize("ov", [0, 2])
def test_u1_sketched_expand_keeps_the_state_and_sorted_bond(right, ov):
    L_, pos = 8, 3
    H = O.heisenberg_XXX(L_, dtype=np.float64, u1=True)
    As, qb = HU.random_u1_tensors(L_, 4, 21, 0, np.float64)
    psi = P.finite_mps_from_tensors(As, charges=(qb, O.SPIN_HALF_CHARGES))
    psi.center = pos if right else pos + 1
    v0 = _dense_state(psi)
    envs = P.FiniteEnvironments(psi, H)
    b = pos + 1 if right else pos
    n0 = len(psi.qb[b])
    P.sketched_expand(pos, right, psi, H, envs, P.SketchedExpand(3, oversampling=ov, seed=4))
    v1 = _dense_state(psi)
    assert np.linalg.norm(v1 / np.linalg.norm(v1) - v0 / np.linalg.norm(v0)) < 1e-12
    q = psi.qb[b]
    assert len(q) > n0 and np.all(np.diff(q) >= 0)
    A = psi.AR[pos + 1] if right else psi.AL[pos - 1]
    ql, qr = (q, psi.qb[pos + 2]) if right else (psi.qb[pos - 1], q)
    assert np.all(A[~HU.block_mask(ql, psi.qp, qr)] == 0)
    m = A.reshape(A.shape[0], -1, order="F") if right else A.reshape(-1, A.shape[2], order="F")
    g = m @ m.conj().T if right else m.conj().T @ m
    assert np.abs(g - np.eye(len(g))).max() < 1e-12


def test_u1_single_site_dmrg_with_sketched_expand_reaches_ed():
    L_ = 10
    As, qb = HU.random_u1_tensors(L_, 2, 5, 0, np.float64)
    H = O.heisenberg_XXX(L_, dtype=np.float64, u1=True)
    psi = P.finite_mps_from_tensors(As, charges=(qb, O.SPIN_HALF_CHARGES))
    alg = P.DMRG(tol=1e-10, maxiter=12, alg_expand=P.SketchedExpand(4, seed=3))
    psi, envs, eps, hist = P.find_groundstate_dmrg(psi, H, alg)
    e_ed = M.ed_ground_energy(L_, 2, M.heisenberg_terms(L_, dtype=np.float64))[0]
    assert -1e-12 * abs(e_ed) <= hist[-1][1] - e_ed < 1e-9 * abs(e_ed), (hist[-1], e_ed)


def test_u1_changebonds_keeps_the_state_and_the_block_structure():
    """changebonds! with SketchedExpand on a U(1) state (sketchedexpand.jl:165-173): bonds
    grow, stay sorted by charge, the tensors stay block sparse and the state is unchanged."""
    L_ = 8
    H = O.heisenberg_XXX(L_, dtype=np.float64, u1=True)
    As, qb = HU.random_u1_tensors(L_, 3, 8, 0, np.float64)
    psi = P.finite_mps_from_tensors(As, charges=(qb, O.SPIN_HALF_CHARGES))
    psi.center = 0
    v0 = _dense_state(psi)
    n0 = sum(len(q) for q in psi.qb)
    psi, _ = P.changebonds(psi, H, P.SketchedExpand(2, seed=5))
    assert psi.center == L_ - 1 and sum(len(q) for q in psi.qb) > n0
    v1 = _dense_state(psi)
    assert abs(abs(np.vdot(v0, v1)) / (np.linalg.norm(v0) * np.linalg.norm(v1)) - 1) < 1e-12
    for b in range(L_ - 1):
        assert np.all(np.diff(psi.qb[b + 1]) >= 0)
        A = psi.AL[b]
        assert np.all(A[~HU.block_mask(psi.qb[b], psi.qp, psi.qb[b + 1])] == 0)
