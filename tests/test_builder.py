"""The product's MPOHamiltonian builder reproduces the oracle's restatement of
mpohamiltonian.jl:439-641 exactly (same channels, same Jordan blocks)."""
import numpy as np
import pytest

import mpsgb
from oracle import models as M


@pytest.mark.parametrize("L", [2, 5, 8])
def test_heisenberg(L):
    a = mpsgb.heisenberg_XXX(L)
    b = M.finite_mpo_hamiltonian(L, 2, M.heisenberg_terms(L))
    assert all(np.array_equal(x, y) for x, y in zip(a.W, b.W))


def test_tfim_and_field_terms():
    a = mpsgb.transverse_field_ising(7, g=0.4, dtype=np.float64)
    b = M.finite_mpo_hamiltonian(7, 2, M.tfim_terms(7, g=0.4, dtype=np.float64), dtype=np.float64)
    assert all(np.array_equal(x, y) for x, y in zip(a.W, b.W))


def test_long_range_cylinder():
    a = mpsgb.j1j2_cylinder(3, 4)
    b = M.finite_mpo_hamiltonian(12, 2, M.j1j2_cylinder_terms(3, 4), dtype=np.float64)
    assert [w.shape for w in a.W] == [w.shape for w in b.W]
    assert all(np.allclose(x, y, atol=1e-15) for x, y in zip(a.W, b.W))


@pytest.mark.parametrize("cell", [1, 2, 3])
def test_infinite(cell):
    a = mpsgb.xxz(cell, 1.0, 1.5, infinite=True)
    b = M.infinite_mpo_hamiltonian(cell, 2, M.xxz_terms(cell, 1.0, 1.5, periodic=True))
    assert all(np.array_equal(x, y) for x, y in zip(a.W, b.W))


def test_mpo_reproduces_ed_spectrum():
    """Contracting the product MPO into a dense matrix gives the ED Hamiltonian."""
    L = 5
    H = mpsgb.xxz(L, 1.0, 0.7, hz=0.2)
    T = H.W[0][0]
    for W in H.W[1:]:
        T = np.einsum("...w,wstv->...stv", T, W)
    # T has legs (s0, s0', s1, s1', ..., last w); gather bra and ket legs
    T = T[..., 0]
    perm = [2 * i for i in range(L)] + [2 * i + 1 for i in range(L)]
    Hd = T.transpose(perm).reshape(2 ** L, 2 ** L)
    e = np.linalg.eigvalsh(Hd)[0]
    assert abs(e - M.ed_ground_energy(L, 2, M.xxz_terms(L, 1.0, 0.7, 0.2))[0]) < 1e-12


@pytest.mark.parametrize("cell", [1, 2])
def test_infinite_rotated_xxz(cell):
    """The sublattice-rotated XXZ chain (one-site invariant form of the Neel phase) builds the
    same MPO as the oracle; a field is refused (it would become staggered)."""
    a = mpsgb.xxz(cell, 1.0, 1.5, infinite=True, rotated=True)
    b = M.infinite_mpo_hamiltonian(cell, 2, M.xxz_terms(cell, 1.0, 1.5, periodic=True,
                                                        rotated=True))
    assert all(np.allclose(x, y, atol=1e-15) for x, y in zip(a.W, b.W))
    with pytest.raises(ValueError):
        mpsgb.xxz(cell, 1.0, 1.5, hz=0.1, infinite=True, rotated=True)
