"""The block-sparse U(1) oracle (oracle/blocksparse.py) against the dense oracle: the same
numbers from the charge-conserving blocks alone -- MPO channel charges, both transfers,
the Jordan-form two-site operator (long-range J1-J2 terms AA/CA/AB and nearest-neighbour
IC/BE), and a DMRG2 local update."""
import numpy as np
import pytest

from oracle import blocksparse as B
from oracle import derivatives as odv
from oracle import mps as P

from mpsgb import operators as O
from mpsgb import u1 as HU

QP = O.SPIN_HALF_CHARGES


def _state(model, L_, D, seed):
    """A seeded random U(1) state (total Sz = 0) in right-canonical form (centre bond 0)."""
    H = (O.j1j2_cylinder(4, 3, u1=True) if model == "j1j2"
         else O.heisenberg_XXX(L_, dtype=np.float64, u1=True))
    As, qb = HU.random_u1_tensors(len(H), D, seed, 0, np.float64)
    psi = P.finite_mps_from_tensors(As, charges=(qb, QP))
    return H, psi


@pytest.mark.parametrize("model", ["j1j2", "heisenberg"])
def test_transfers_match_dense(model):
    H, psi = _state(model, 12, 24, 3)
    dq = B.mpo_channel_charges([H.W[i] for i in range(len(H))], QP)
    # a charge-conserving GL / GR of each bond from the dense recursion itself
    GL = np.ones((1, 1, 1))
    for j in range(6):
        A = psi.AR[j]
        ref = odv.transfer_left(GL, H.W[j], A, A)
        got, dq_out = B.transfer_left(GL, H.W[j], A, psi.qb[j], QP, psi.qb[j + 1], dq[j])
        assert np.array_equal(dq_out, dq[j + 1])
        assert np.linalg.norm(got - ref) <= 1e-12 * max(1.0, np.linalg.norm(ref))
        GL = ref
    GR = np.ones((1, 1, 1))
    for j in range(len(H) - 1, 5, -1):
        A = psi.AR[j]
        ref = odv.transfer_right(GR, H.W[j], A, A)
        got = B.transfer_right(GR, H.W[j], A, psi.qb[j], QP, psi.qb[j + 1], dq[j])
        assert np.linalg.norm(got - ref) <= 1e-12 * max(1.0, np.linalg.norm(ref))
        GR = ref


@pytest.mark.parametrize("model", ["j1j2", "heisenberg"])
def test_ac2_operator_matches_dense(model):
    H, psi = _state(model, 12, 40, 5)
    envs = P.FiniteEnvironments(psi, H)
    envb = B.FiniteEnvironmentsU1(psi, H)
    pos = 5
    # right-canonical state: environments left of pos from AL = AR here is not needed; use
    # the dense environments of the right-gauged tensors on both sides
    GL, GR = envs.leftenv(0, psi), envs.rightenv(pos + 1, psi)
    GLb = envb.leftenv(0, psi)
    assert np.array_equal(GL, GLb)
    GRb = envb.rightenv(pos + 1, psi)
    assert np.linalg.norm(GRb - GR) <= 1e-12 * np.linalg.norm(GR)
    # an operator on bond (pos, pos+1) with the right environment of the state and a left
    # environment made by the recursion over the (right-gauged) tensors of sites < pos
    for j in range(pos):
        GL, _ = B.transfer_left(GL, H.W[j], psi.AR[j], psi.qb[j], QP, psi.qb[j + 1], envb.dq[j])
    dense = odv.JordanAC2(GL, H.W[pos], H.W[pos + 1], GR)
    op = B.JordanAC2U1(GL, H.W[pos], H.W[pos + 1], GR, psi.qb[pos], QP, psi.qb[pos + 2],
                       envb.dq[pos], envb.dq[pos + 2])
    assert op.op.terms() == dense.terms()
    if model == "j1j2":
        assert "AA" in dense.terms() and "CA" in dense.terms() and "AB" in dense.terms()
    else:
        assert "IC" in dense.terms() and "BE" in dense.terms()
    rng = np.random.default_rng(9)
    x = rng.standard_normal(op.mask.shape) * op.mask
    ref = dense(x)
    got = op(x)
    assert np.linalg.norm(got - ref) <= 1e-12 * np.linalg.norm(ref)
    assert np.all(got[~op.mask] == 0)
    assert op.block_flops() > 0


def test_dmrg2_local_update_matches_dense():
    H, psi = _state("j1j2", 12, 32, 7)
    pos = 4
    alg = P.DMRG2(maxdim=32, cutoff=1e-10)
    psi_d = psi.copy()
    psi_b = psi.copy()
    envs_d = P.FiniteEnvironments(psi_d, H)
    envs_b = B.FiniteEnvironmentsU1(psi_b, H)
    out = []
    for ps, en, upd in ((psi_d, envs_d, P.dmrg2_local_update),
                        (psi_b, envs_b, B.dmrg2_local_update)):
        stats = {"matvecs": 0}
        res = None
        for p in range(pos + 1):
            res = upd(p, True, ps, H, alg, en, 1.0, 0.0, 0.5, stats)
        out.append(res)
    (el_d, et_d, _, val_d), (el_b, et_b, _, val_b) = out
    assert abs(val_d - val_b) <= 1e-10 * abs(val_d)
    assert abs(el_d - el_b) <= 1e-8 * max(el_d, 1e-6)
    assert np.array_equal(psi_d.qb[pos + 1], psi_b.qb[pos + 1])


def test_blockwise_canonical_form_matches_dense():
    H = O.heisenberg_XXX(10, dtype=np.float64, u1=True)
    As, qb = HU.random_u1_tensors(10, 24, 13, 0, np.float64)
    ref = P.finite_mps_from_tensors(As, charges=(qb, QP))
    got = B.canonical_u1(As, qb, QP, 0)
    for i in range(10):
        assert np.linalg.norm(got.AR[i] - ref.AR[i]) <= 1e-12 * np.linalg.norm(ref.AR[i])
        assert np.linalg.norm(got.AL[i] - ref.AL[i]) <= 1e-12 * np.linalg.norm(ref.AL[i])
    assert abs(abs(got.C[0].ravel()[0]) - abs(ref.C[0].ravel()[0])) < 1e-12
