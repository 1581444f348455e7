"""MPOHamiltonian linear algebra (src/operators/mpohamiltonian.jl:741-820): the Jordan-block
sum H1 + H2, scaling and subtraction, checked on the dense matrices of finite chains and on
the block structure of infinite ones."""
import numpy as np
import pytest

import mpsgb
from oracle import models as M


def _matrix(H):
    """The d^L x d^L matrix of a finite Jordan MPO (first site one left channel, last site
    one right channel)."""
    T = H.W[0][0]
    for w in H.W[1:]:
        T = np.tensordot(T, w, axes=([-1], [0]))
    T = T[..., 0]
    L_ = len(H.W)
    d = H.W[0].shape[1]
    perm = [2 * i for i in range(L_)] + [2 * i + 1 for i in range(L_)]
    return T.transpose(perm).reshape(d ** L_, d ** L_)


@pytest.mark.parametrize("u1", [False, True])
def test_sum_scale_and_difference_are_linear(u1):
    L_ = 5
    H1 = mpsgb.heisenberg_XXX(L_, dtype=np.float64, u1=u1)
    H2 = mpsgb.xxz(L_, 1.0, 0.4, 0.3, dtype=np.float64, u1=u1)
    A, B = _matrix(H1), _matrix(H2)
    assert np.abs(_matrix(H1 + H2) - (A + B)).max() < 1e-13
    assert np.abs(_matrix(2.5 * H1) - 2.5 * A).max() < 1e-13
    assert np.abs(_matrix(H1 - 0.5 * H2) - (A - 0.5 * B)).max() < 1e-13
    # the spectrum of the sum is that of the lattice terms' sum
    terms = M.heisenberg_terms(L_, dtype=np.float64) + M.xxz_terms(L_, 1.0, 0.4, 0.3,
                                                                   dtype=np.float64)
    Hm = M.ed_hamiltonian(L_, 2, terms)
    e = np.linalg.eigvalsh(Hm.toarray() if hasattr(Hm, "toarray") else Hm)
    assert np.abs(np.linalg.eigvalsh(_matrix(H1 + H2)) - e).max() < 1e-12
    S = H1 + H2
    assert len(S.chans) == L_ + 1 and S.chans[0] == [1] and S.chans[-1] == [1]
    assert all(sum(c) == S.W[i].shape[0] for i, c in enumerate(S.chans[:-1]))


def test_infinite_sum_keeps_the_jordan_blocks():
    H1 = mpsgb.transverse_field_ising(1, g=0.8, infinite=True)
    H2 = mpsgb.heisenberg_XXX(1, infinite=True)
    S = H1 + H2
    w1, w2, w = H1.W[0], H2.W[0], S.W[0]
    n1, n2 = w1.shape[0] - 2, w2.shape[0] - 2
    assert w.shape[0] == w.shape[3] == 2 + n1 + n2
    I = np.eye(w1.shape[1])
    assert np.allclose(w[0, :, :, 0], I) and np.allclose(w[-1, :, :, -1], I)
    assert np.allclose(w[0, :, :, -1], w1[0, :, :, -1] + w2[0, :, :, -1])          # D
    assert np.allclose(w[0, :, :, 1:1 + n1], w1[0, :, :, 1:-1])                     # C
    assert np.allclose(w[0, :, :, 1 + n1:-1], w2[0, :, :, 1:-1])
    assert np.allclose(w[1 + n1:-1, :, :, 1 + n1:-1], w2[1:-1, :, :, 1:-1])         # A
    assert np.allclose(w[1:1 + n1, :, :, 1 + n1:-1], 0)
    assert np.allclose(w[1 + n1:-1, :, :, -1], w2[1:-1, :, :, -1])                  # B


def test_onsite_shift():
    L_ = 4
    H = mpsgb.heisenberg_XXX(L_, dtype=np.float64)
    lam = np.array([0.1, -0.2, 0.3, 0.05])
    A = _matrix(H)
    assert np.abs(_matrix(H + lam) - (A + lam.sum() * np.eye(A.shape[0]))).max() < 1e-13
    assert np.abs(_matrix(H - 0.7) - (A - 0.7 * L_ * np.eye(A.shape[0]))).max() < 1e-13
    assert np.abs(_matrix(0.7 + H) - (A + 0.7 * L_ * np.eye(A.shape[0]))).max() < 1e-13


@pytest.mark.parametrize("u1", [False, True])
def test_product_is_the_operator_product(u1):
    L_ = 4
    H1 = mpsgb.heisenberg_XXX(L_, dtype=np.float64, u1=u1)
    H2 = mpsgb.xxz(L_, 1.0, 0.4, 0.3, dtype=np.float64, u1=u1)
    P_ = H1 * H2
    assert np.abs(_matrix(P_) - _matrix(H1) @ _matrix(H2)).max() < 1e-12
    assert all(sum(c) == P_.W[i].shape[0] for i, c in enumerate(P_.chans[:-1]))
    # upper triangular channel structure, identity corners
    w = P_.W[1]
    I = np.eye(2)
    assert np.allclose(w[0, :, :, 0], I) and np.allclose(w[-1, :, :, -1], I)
    for a in range(w.shape[0]):
        for b in range(a):
            assert np.all(w[a, :, :, b] == 0)
