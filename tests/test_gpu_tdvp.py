"""Single-site TDVP on the device (timestep!, tdvp.jl:135-211) against the oracle."""
import numpy as np
import pytest

import mpsgb
from oracle import models as M
from oracle import mps as P

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    return mpsgb.context(0)


def test_tdvp_real_time_matches_oracle(ctx):
    L_, D, dt = 8, 8, 0.05
    terms = M.xxz_terms(L_, 1.0, 0.6, 0.3)
    As = P.random_initial_tensors(L_, 2, D, 13)
    oH = M.finite_mpo_hamiltonian(L_, 2, terms)
    opsi = P.finite_mps_from_tensors(As)
    oenvs = P.FiniteEnvironments(opsi, oH)
    e0 = P.expectation_value(opsi, oH, oenvs, 0)
    H = mpsgb.xxz(L_, 1.0, 0.6, 0.3)
    psi = mpsgb.FiniteMPS.from_tensors(As, ctx)
    envs = mpsgb.FiniteEnvironments(psi, H)
    alg = mpsgb.TDVP()
    for k in range(3):
        opsi, oenvs = P.tdvp_timestep(opsi, oH, oenvs, k * dt, dt)
        psi, envs = mpsgb.timestep(psi, H, k * dt, dt, alg, envs)
    a, b = psi.ac(0).numpy(), opsi.ac(0)
    assert np.linalg.norm(a - b) / np.linalg.norm(b) < 1e-9
    for i in range(1, L_):
        assert np.allclose(psi.AR[i].numpy(), opsi.AR[i], atol=1e-9)
    e = mpsgb.expectation_value(psi, H, envs, 0)
    assert abs(e - e0) < 1e-9          # 1-site TDVP conserves energy
    assert abs(np.linalg.norm(a) - 1.0) < 1e-10


def test_tdvp_imaginary_time_lowers_energy(ctx):
    L_ = 8
    H = mpsgb.heisenberg_XXX(L_)
    psi = mpsgb.FiniteMPS.random(L_, 2, 16, 21, np.complex128, ctx)
    envs = mpsgb.FiniteEnvironments(psi, H)
    alg = mpsgb.TDVP()
    e_prev = mpsgb.expectation_value(psi, H, envs, 0)
    for k in range(4):
        psi, envs = mpsgb.timestep(psi, H, 0.0, 0.2, alg, envs, imaginary_evolution=True)
        psi.ac_tensor.normalize_()
        e = mpsgb.expectation_value(psi, H, envs, 0)
        assert e < e_prev + 1e-12
        e_prev = e
