"""The channel-assignment MPO builder (mpohamiltonian.jl:349-519) against the identities of
the reference's own MPOHamiltonian tests (test/operators/mpohamiltonian.jl:77-150): the dense
operator of onsite, nearest-neighbour and longer-range terms, repeated terms adding up, and
the linear algebra of Hamiltonians -- real and complex, random Hermitian operators."""
import numpy as np
import pytest

from mpsgb.operators import FiniteMPOHamiltonian


def _matrix(H):
    T = H.W[0][0]
    for w in H.W[1:]:
        T = np.tensordot(T, w, axes=([-1], [0]))
    T = T[..., 0]
    L_ = len(H.W)
    d = H.W[0].shape[1]
    perm = [2 * i for i in range(L_)] + [2 * i + 1 for i in range(L_)]
    return T.transpose(perm).reshape(d ** L_, d ** L_)


def _embed(op, sites, L_, d):
    """The d^L x d^L matrix of `op` (one-site (d, d) or two-site (d, d, d, d) with legs
    (s_i, s_j, s_i', s_j')) acting on `sites` of an L-site chain (site 0 most significant)."""
    n = len(sites)
    full = np.eye(d ** L_, dtype=op.dtype).reshape([d] * (2 * L_))
    o = op.reshape([d] * (2 * n))
    # contract op's input legs with the identity's output legs of those sites
    out_axes = list(sites)
    res = np.tensordot(o, full, axes=(list(range(n, 2 * n)), out_axes))
    # the op's output legs now lead; move them back to the site positions
    res = np.moveaxis(res, list(range(n)), list(sites))
    return res.reshape(d ** L_, d ** L_)


def _rand_herm(rng, shape, dt):
    a = rng.standard_normal(shape)
    if np.dtype(dt).kind == "c":
        a = a + 1j * rng.standard_normal(shape)
    m = a.reshape(int(np.prod(shape[:len(shape) // 2])), -1)
    m = m + m.conj().T
    return m.reshape(shape).astype(dt)


@pytest.mark.parametrize("dt", [np.float64, np.complex128])
def test_builder_matches_the_dense_operators(dt):
    rng = np.random.default_rng(11)
    L_, d = 3, 2
    O1 = _rand_herm(rng, (d, d), dt)
    O2 = _rand_herm(rng, (d, d, d, d), dt)
    H1 = FiniteMPOHamiltonian(L_, d, [((i,), O1) for i in range(L_)], dt)
    H2 = FiniteMPOHamiltonian(L_, d, [((i, i + 1), O2) for i in range(L_ - 1)], dt)
    H3 = FiniteMPOHamiltonian(L_, d, [((0,), O1), ((1, 2), O2), ((0, 2), O2)], dt)
    assert np.allclose(_matrix(H1), sum(_embed(O1, (i,), L_, d) for i in range(L_)), atol=1e-12)
    assert np.allclose(_matrix(H2), sum(_embed(O2, (i, i + 1), L_, d) for i in range(L_ - 1)),
                       atol=1e-12)
    ref3 = _embed(O1, (0,), L_, d) + _embed(O2, (1, 2), L_, d) + _embed(O2, (0, 2), L_, d)
    assert np.allclose(_matrix(H3), ref3, atol=1e-12)
    # repeated terms add up
    H4 = FiniteMPOHamiltonian(L_, d, [((i,), O1 / 2) for i in range(L_)] * 2, dt)
    assert np.allclose(_matrix(H4), _matrix(H1), atol=1e-12)
    H5 = FiniteMPOHamiltonian(L_, d, [((i, i + 1), O2 / 2) for i in range(L_ - 1)] * 2, dt)
    assert np.allclose(_matrix(H5), _matrix(H2), atol=1e-12)
    # linear algebra
    Hs = [FiniteMPOHamiltonian(L_, d, [((i,), O1)], dt) for i in range(L_)]
    assert np.allclose(_matrix(Hs[0] + Hs[1] + Hs[2]), _matrix(H1), atol=1e-12)
    assert np.allclose(_matrix(0.8 * H1 + 0.2 * H1), _matrix(H1), atol=1e-12)
    assert np.allclose(_matrix(H1 + H2), _matrix(H1) + _matrix(H2), atol=1e-12)
