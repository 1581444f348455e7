"""VUMPS and InfiniteMPOHamiltonian environments on the device against the oracle."""
import numpy as np
import pytest

import mpsgb
from oracle import models as M
from oracle import vumps as V

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    return mpsgb.context(0)


def _A(D, seed):
    rng = np.random.default_rng(seed)
    return rng.standard_normal((D, 2, D)) + 1j * rng.standard_normal((D, 2, D))


def test_gauge_fixing_matches_oracle(ctx):
    A = _A(10, 3)
    opsi = V.infinite_mps(A)
    psi = mpsgb.InfiniteMPS.from_tensor(A, ctx)
    AL, AR, C = psi.to_numpy()
    assert np.allclose(AL, opsi.AL, atol=1e-10)
    assert np.allclose(AR, opsi.AR, atol=1e-10)
    assert np.allclose(C, opsi.C, atol=1e-10)


@pytest.mark.parametrize("model", ["tfim", "xxz_field"])
def test_infinite_environments_match_oracle(ctx, model):
    if model == "tfim":
        terms = M.tfim_terms(1, g=0.8, periodic=True)
        H = mpsgb.transverse_field_ising(1, g=0.8, infinite=True)
    else:
        terms = M.xxz_terms(1, 1.0, 0.5, 0.3, periodic=True)
        H = mpsgb.xxz(1, 1.0, 0.5, 0.3, infinite=True)
    oH = M.infinite_mpo_hamiltonian(1, 2, terms)
    A = _A(8, 4)
    opsi = V.infinite_mps(A)
    GL, GR = V.infinite_envs(opsi, oH[0], oH.chans[0], tol=1e-13)
    psi = mpsgb.InfiniteMPS.from_tensor(A, ctx)
    envs = mpsgb.InfiniteEnvironments(psi, H).recalculate(psi, tol=1e-13)
    assert np.allclose(envs.GL.numpy(), GL, atol=1e-9)
    assert np.allclose(envs.GR.numpy(), GR, atol=1e-9)
    e_dev = mpsgb.infinite.energy_density(psi, envs)
    assert abs(e_dev - V.energy_density(opsi, oH[0], GL, GR)) < 1e-10


def test_vumps_tfim_reaches_closed_form(ctx):
    g = 0.5
    H = mpsgb.transverse_field_ising(1, g=g, infinite=True)
    psi = mpsgb.InfiniteMPS.from_tensor(_A(12, 1), ctx)
    psi, envs, eps, hist = mpsgb.find_groundstate_vumps(psi, H, mpsgb.VUMPS(tol=1e-10, maxiter=100))
    assert eps <= 1e-10
    assert abs(hist[-1]["energy"] - M.tfim_infinite_energy_density(g)) < 1e-11


@pytest.mark.parametrize("imaginary", [False, True])
def test_infinite_tdvp_matches_oracle(ctx, imaginary):
    """Three one-site TDVP steps of an InfiniteMPS (real and imaginary time) against the
    oracle: the same gauge-fixed tensors and energy density."""
    g = 0.8
    terms = M.tfim_terms(1, g=g, periodic=True)
    oH = M.infinite_mpo_hamiltonian(1, 2, terms)
    H = mpsgb.transverse_field_ising(1, g=g, infinite=True)
    A = _A(8, 5)
    opsi = V.infinite_mps(A)
    psi = mpsgb.InfiniteMPS.from_tensor(A, ctx)
    alg = mpsgb.TDVP(integrator=mpsgb.Lanczos(krylovdim=30, maxiter=200, tol=1e-12))
    GL = GR = None
    envs = None
    for _ in range(3):
        opsi, GL, GR = V.tdvp_timestep_infinite(opsi, oH, 0.05, GL, GR, imaginary=imaginary)
        psi, envs = mpsgb.timestep_infinite(psi, H, 0.0, 0.05, alg, envs,
                                            imaginary_evolution=imaginary)
    AL, AR, C = psi.to_numpy()
    assert np.allclose(AL, opsi.AL, atol=1e-8)
    assert np.allclose(C, opsi.C, atol=1e-8)
    e = mpsgb.infinite.energy_density(psi, envs)
    assert abs(e - V.energy_density(opsi, oH[0], GL, GR)) < 1e-9


def test_infinite_imaginary_time_approaches_ground_state(ctx):
    g = 0.5
    H = mpsgb.transverse_field_ising(1, g=g, infinite=True)
    psi = mpsgb.InfiniteMPS.from_tensor(_A(8, 6), ctx)
    alg = mpsgb.TDVP(integrator=mpsgb.Lanczos(krylovdim=30, maxiter=200, tol=1e-12))
    envs = None
    for _ in range(60):
        psi, envs = mpsgb.timestep_infinite(psi, H, 0.0, 0.2, alg, envs, imaginary_evolution=True)
    e = mpsgb.infinite.energy_density(psi, envs)
    assert abs(e - M.tfim_infinite_energy_density(g)) < 1e-7


def test_vumps_rotated_xxz_neel_phase(ctx):
    """XXZ with Jxy = 1, Jz = 1.5 after the sublattice rotation: one-site VUMPS on the
    device converges to the oracle's state energy and sits just above the Bethe-ansatz
    energy density (D = 24)."""
    delta = 1.5
    terms = M.xxz_terms(1, 1.0, delta, periodic=True, rotated=True)
    oH = M.infinite_mpo_hamiltonian(1, 2, terms)
    H = mpsgb.xxz(1, 1.0, delta, 0.0, infinite=True, rotated=True)
    A = _A(24, 7)
    _, _, _, oeps, ohist = V.vumps(V.infinite_mps(A), oH, tol=1e-10, maxiter=100)
    psi = mpsgb.InfiniteMPS.from_tensor(A, ctx)
    psi, envs, eps, hist = mpsgb.find_groundstate_vumps(psi, H, mpsgb.VUMPS(tol=1e-10,
                                                                            maxiter=100))
    assert eps <= 1e-9 and oeps <= 1e-9
    e = hist[-1]["energy"]
    assert abs(e - ohist[-1][1]) < 1e-10
    de = e - M.xxz_infinite_energy_density(delta)
    assert 0.0 <= de < 1e-6


@pytest.mark.parametrize("model", ["tfim", "xxz_rotated"])
def test_idmrg_matches_oracle(ctx, model):
    """One-site IDMRG (idmrg.jl:194-228) on the device against the oracle from the same
    initial state: the same iteration count, converged energy density and gauge tensors."""
    if model == "tfim":
        terms = M.tfim_terms(1, g=0.5, periodic=True)
        H = mpsgb.transverse_field_ising(1, g=0.5, infinite=True)
        exact, maxiter = M.tfim_infinite_energy_density(0.5), 200
    else:
        terms = M.xxz_terms(1, 1.0, 3.0, periodic=True, rotated=True)
        H = mpsgb.xxz(1, 1.0, 3.0, 0.0, infinite=True, rotated=True)
        exact, maxiter = M.xxz_infinite_energy_density(3.0), 30
    oH = M.infinite_mpo_hamiltonian(1, 2, terms)
    A = _A(12, 1)
    opsi, GL, GR, oeps, ohist = V.idmrg(V.infinite_mps(A), oH, tol=1e-10, maxiter=maxiter)
    oe = V.energy_density(opsi, oH[0], GL, GR)
    psi = mpsgb.InfiniteMPS.from_tensor(A, ctx)
    psi, envs, eps, hist = mpsgb.find_groundstate_idmrg(psi, H, mpsgb.IDMRG(tol=1e-10,
                                                                            maxiter=maxiter))
    e = mpsgb.infinite.energy_density(psi, envs)
    assert abs(e - oe) < 1e-10
    assert 0.0 <= e - exact < 1e-7
    if model == "tfim":
        assert eps <= 1e-10 and len(hist) == len(ohist)
        AL, AR, C = psi.to_numpy()
        assert np.allclose(C, opsi.C, atol=1e-8)
