"""InfiniteMPS with a two-site unit cell on the device (VUMPS, IDMRG2) against the
oracle's unit-cell restatement (oracle/cell.py)."""
import numpy as np
import pytest

import mpsgb
from mpsgb import cell as GC
from oracle import cell as Ce
from oracle import models as M

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    return mpsgb.context(0)


def _As(D, n, seed):
    rng = np.random.default_rng(seed)
    return [rng.standard_normal((D, 2, D)) + 1j * rng.standard_normal((D, 2, D))
            for _ in range(n)]


def test_cell_gauge_and_vumps_match_oracle(ctx):
    """Gauge fixing of a two-site cell and two-site VUMPS on the TFIM (g = 0.5): the same
    gauge tensors and the same converged energy per site as the oracle."""
    As = _As(10, 2, 21)
    opsi = Ce.infinite_mps(As)
    psi = GC.InfiniteMPSCell.from_tensors(As, ctx)
    AL, AR, C = psi.to_numpy()
    for s in range(2):
        assert np.allclose(AL[s], opsi.AL[s], atol=1e-10)
        assert np.allclose(AR[s], opsi.AR[s], atol=1e-10)
        assert np.allclose(C[s], opsi.C[s], atol=1e-10)
    oH = M.infinite_mpo_hamiltonian(2, 2, M.tfim_terms(2, g=0.5, periodic=True))
    H = mpsgb.transverse_field_ising(2, g=0.5, infinite=True)
    _, _, _, oeps, ohist = Ce.vumps(opsi, oH, tol=1e-10, maxiter=50)
    psi, envs, eps, hist = GC.find_groundstate_vumps(psi, H, mpsgb.VUMPS(tol=1e-10, maxiter=50))
    assert eps <= 1e-9 and oeps <= 1e-9
    assert abs(hist[-1]["energy"] - ohist[-1][1]) < 1e-10
    assert abs(hist[-1]["energy"] - M.tfim_infinite_energy_density(0.5)) < 1e-10


def test_idmrg2_matches_oracle(ctx):
    """IDMRG2 on a two-site TFIM cell from D = 4 under truncrank(16): the same iteration
    count and energy as the oracle, at the free-fermion energy density."""
    As = _As(4, 2, 22)
    oH = M.infinite_mpo_hamiltonian(2, 2, M.tfim_terms(2, g=0.5, periodic=True))
    H = mpsgb.transverse_field_ising(2, g=0.5, infinite=True)
    opsi, GL, GR, oeps, ohist = Ce.idmrg2(Ce.infinite_mps(As), oH, maxdim=16, atol=1e-10,
                                          tol=1e-10, maxiter=50)
    psi = GC.InfiniteMPSCell.from_tensors(As, ctx)
    psi, envs, eps, hist = GC.find_groundstate_idmrg2(
        psi, H, GC.IDMRG2(maxdim=16, cutoff=1e-10, tol=1e-10, maxiter=50))
    e = GC.energy(psi, envs) / 2
    assert eps <= 1e-9
    assert abs(len(hist) - len(ohist)) <= 1
    assert abs(e - Ce.energy(opsi, oH, GL, GR) / 2) < 1e-10
    assert abs(e - M.tfim_infinite_energy_density(0.5)) < 1e-9


def test_idmrg_on_a_cell_matches_oracle(ctx):
    """IDMRG (one-site updates, idmrg.jl:85-229) on a two-site TFIM cell at D = 6: the same
    iteration count, energy changes and final energy per site as the oracle's cell
    restatement."""
    As = _As(6, 2, 23)
    oH = M.infinite_mpo_hamiltonian(2, 2, M.tfim_terms(2, g=0.9, periodic=True))
    H = mpsgb.transverse_field_ising(2, g=0.9, infinite=True)
    opsi, GL, GR, oeps, ohist = Ce.idmrg1(Ce.infinite_mps(As), oH, tol=1e-9, maxiter=200)
    psi = GC.InfiniteMPSCell.from_tensors(As, ctx)
    psi, envs, eps, hist = GC.find_groundstate_idmrg(psi, H, mpsgb.IDMRG(tol=1e-9, maxiter=200))
    assert eps <= 1e-9 and oeps <= 1e-9
    assert abs(len(hist) - len(ohist)) <= 1
    assert abs(np.real(hist[-1]["energy_change"]) - ohist[-1][1]) < 1e-8
    assert abs(GC.energy(psi, envs) / 2 - Ce.energy(opsi, oH, GL, GR) / 2) < 1e-10


def test_tdvp_step_on_a_cell_matches_oracle(ctx):
    """One real-time TDVP step of a two-site cell (tdvp.jl:72-133): the same AL, C and
    energy as the oracle's cell restatement."""
    As = _As(6, 2, 24)
    oH = M.infinite_mpo_hamiltonian(2, 2, M.tfim_terms(2, g=0.7, periodic=True))
    H = mpsgb.transverse_field_ising(2, g=0.7, infinite=True)
    op2, GL, GR = Ce.tdvp_timestep(Ce.infinite_mps(As), oH, 0.05)
    p2, envs = GC.timestep(GC.InfiniteMPSCell.from_tensors(As, ctx), H, 0.0, 0.05)
    AL, AR, C = p2.to_numpy()
    for s in range(2):
        assert np.abs(AL[s] - op2.AL[s]).max() < 1e-8, s
        assert np.abs(C[s] - op2.C[s]).max() < 1e-8, s
    assert abs(GC.energy(p2, envs) - Ce.energy(op2, oH, GL, GR)) < 1e-9
