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
