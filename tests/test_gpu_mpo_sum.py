"""A summed MPOHamiltonian (mpohamiltonian.jl:741-786) on the device: the two-site operator of
H1 + H2 applies as the sum of the two operators (the linearity the reference tests for LazySum,
test/operators/lazysum.jl:79-260), and DMRG2 on a U(1) sum reaches exact diagonalisation."""
import numpy as np
import pytest

import mpsgb
from mpsgb import u1 as HU
from mpsgb.operators import SPIN_HALF_CHARGES as QP
from oracle import models as M

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    return mpsgb.context(0)


def test_sum_operator_is_the_sum_of_operators(ctx):
    L_, pos = 8, 3
    H1 = mpsgb.heisenberg_XXX(L_, dtype=np.float64)
    H2 = mpsgb.transverse_field_ising(L_, g=0.7, dtype=np.float64)
    S = H1 + 0.5 * H2
    rng = np.random.default_rng(7)
    bond = lambda b: min(2 ** b, 8, 2 ** (L_ - b))
    As = [rng.standard_normal((bond(i), 2, bond(i + 1))) for i in range(L_)]
    psi = mpsgb.FiniteMPS.from_tensors(As, ctx, center=pos)
    x = mpsgb.ac2_from(psi.ac(pos), psi.AR[pos + 1])
    ac, c = psi.ac(pos), psi.C[pos]
    ys = {"AC2": [], "AC": [], "C": []}
    for H in (S, H1, H2):
        envs = mpsgb.FiniteEnvironments(psi, H)
        ys["AC2"].append(mpsgb.AC2_hamiltonian(pos, psi, H, envs)(x).numpy())
        ys["AC"].append(mpsgb.AC_hamiltonian(pos, psi, H, envs)(ac).numpy())
        ys["C"].append(mpsgb.C_hamiltonian(pos - 1, psi, H, envs)(c).numpy())
    for kind, (y_sum, y1, y2) in ys.items():
        ref = y1 + 0.5 * y2
        assert np.linalg.norm(y_sum - ref) <= 1e-12 * np.linalg.norm(ref), kind


def test_u1_dmrg2_on_a_sum_reaches_ed(ctx):
    L_ = 10
    H = mpsgb.heisenberg_XXX(L_, dtype=np.float64, u1=True) + \
        mpsgb.xxz(L_, 0.0, 1.0, 0.0, dtype=np.float64, u1=True) * 0.3
    terms = M.heisenberg_terms(L_, dtype=np.float64) + [
        (s, 0.3 * op) for s, op in M.xxz_terms(L_, 0.0, 1.0, 0.0, dtype=np.float64)]
    e_ed = M.ed_ground_energy(L_, 2, terms)[0]
    As, qb = HU.random_u1_tensors(L_, 16, 3, 0, np.float64)
    psi = mpsgb.FiniteMPS.from_tensors(As, ctx, charges=(qb, QP))
    psi, envs, eps, hist = mpsgb.find_groundstate(psi, H, mpsgb.DMRG2(maxdim=32, cutoff=1e-12),
                                                  maxsweeps=6)
    assert abs(hist[-1]["energy"] - e_ed) < 1e-9 * abs(e_ed), (hist[-1], e_ed)


def _matrix(H):
    T = H.W[0][0]
    for w in H.W[1:]:
        T = np.tensordot(T, w, axes=([-1], [0]))
    T = T[..., 0]
    L_ = len(H.W)
    d = H.W[0].shape[1]
    perm = [2 * i for i in range(L_)] + [2 * i + 1 for i in range(L_)]
    return T.transpose(perm).reshape(d ** L_, d ** L_)


@pytest.mark.parametrize("dt", [np.float64, np.complex128])
def test_variance_matches_the_dense_state(ctx, dt):
    """variance(::FiniteMPS, H) (toolbox.jl:125-128) through the MPO product H * H."""
    L_ = 6
    H = mpsgb.transverse_field_ising(L_, g=0.8, dtype=dt)
    rng = np.random.default_rng(9)
    bond = lambda b: min(2 ** b, 4, 2 ** (L_ - b))
    As = [rng.standard_normal((bond(i), 2, bond(i + 1))).astype(dt) for i in range(L_)]
    psi = mpsgb.FiniteMPS.from_tensors(As, ctx)
    v = mpsgb.variance(psi, H)
    T = psi.C[0].numpy()
    for i in range(L_):
        T = np.tensordot(T, psi.AR[i].numpy(), axes=([-1], [0]))
    vec = T.reshape(-1)
    Hm = _matrix(H)
    nrm = np.vdot(vec, vec).real
    e = np.vdot(vec, Hm @ vec).real / nrm
    e2 = np.vdot(Hm @ vec, Hm @ vec).real / nrm
    assert abs(v - (e2 - e * e)) <= 1e-10 * max(1.0, e2), (v, e2 - e * e)
