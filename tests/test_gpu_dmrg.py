"""End-to-end DMRG on the device against the oracle and the reference's known answers."""
import json
import os

import numpy as np
import pytest

import mpsgb
from oracle import models as M
from oracle import mps as P

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
KAT = json.load(open(os.path.join(HERE, "golden", "known_answers.json")))


@pytest.fixture(scope="module")
def ctx():
    return mpsgb.context(0)


def test_tfim_doctest_known_answer(ctx):
    L_ = 4
    X = np.array([[0, 1], [1, 0]], dtype=np.float64)
    Z = np.array([[1, 0], [0, -1]], dtype=np.float64)
    terms = [((i, i + 1), -np.einsum("ik,jl->ijkl", X, X)) for i in range(L_ - 1)]
    terms += [((i,), -Z) for i in range(L_)]
    H = mpsgb.FiniteMPOHamiltonian(L_, 2, terms, dtype=np.float64)
    psi = mpsgb.FiniteMPS.from_tensors([np.ones((1, 2, 1)) for _ in range(L_)], ctx)
    psi, envs, eps, hist = mpsgb.find_groundstate(psi, H, mpsgb.DMRG2(maxdim=16), maxsweeps=30)
    assert round(hist[-1]["energy"], 4) == KAT["tfim_L4_doctest"]["energy_rounded_4"]


def test_dmrg2_matches_oracle_fp64(ctx):
    L_, D = 12, 16
    terms = M.heisenberg_terms(L_)
    As = P.random_initial_tensors(L_, 2, D, 99)
    oH = M.finite_mpo_hamiltonian(L_, 2, terms)
    _, _, _, ohist = P.find_groundstate_dmrg2(P.finite_mps_from_tensors(As), oH,
                                              P.DMRG2(maxdim=D, cutoff=1e-10), maxsweeps=6)
    H = mpsgb.heisenberg_XXX(L_)
    psi = mpsgb.FiniteMPS.from_tensors(As, ctx)
    psi, envs, eps, hist = mpsgb.find_groundstate(psi, H, mpsgb.DMRG2(maxdim=D, cutoff=1e-10),
                                                  maxsweeps=6)
    for a, b in zip(hist, ohist):
        assert abs(a["energy"] - b[1]) < 1e-10 * abs(b[1]), (a, b)
    e_ed = M.ed_ground_energy(L_, 2, terms)[0]
    assert abs(hist[-1]["energy"] - e_ed) < 1e-6


def test_heisenberg_L20_known_answer(ctx):
    L_ = 20
    H = mpsgb.heisenberg_XXX(L_, dtype=np.float64)
    psi = mpsgb.FiniteMPS.random(L_, 2, 8, 5, np.float64, ctx)
    psi, envs, eps, hist = mpsgb.find_groundstate(psi, H, mpsgb.DMRG2(maxdim=48, cutoff=1e-12),
                                                  maxsweeps=12)
    kat = KAT["heisenberg_L20_spin_half"]
    assert abs(hist[-1]["energy"] - kat["energy"]) < kat["atol"]


def test_dmrg1_matches_ed(ctx):
    L_ = 8
    terms = M.xxz_terms(L_, 1.0, 0.8, 0.2)
    H = mpsgb.xxz(L_, 1.0, 0.8, 0.2)
    psi = mpsgb.FiniteMPS.random(L_, 2, 16, 3, np.complex128, ctx)
    psi, envs, eps, hist = mpsgb.find_groundstate(psi, H, mpsgb.DMRG(), maxsweeps=12)
    e_ed = M.ed_ground_energy(L_, 2, terms)[0]
    assert abs(mpsgb.expectation_value(psi, H, envs, 0) - e_ed) < 1e-8


def test_dmrg2_split_precision_energy(ctx):
    """bf16x3 contractions with FP64 Krylov/gauge: the converged energy agrees with the
    FP64 device path (energy error is second order in the contraction error)."""
    L_, D = 16, 32
    H = mpsgb.heisenberg_XXX(L_, dtype=np.float64)
    res = {}
    for prec in ("fp64", "bf16x3"):
        psi = mpsgb.FiniteMPS.random(L_, 2, D, 17, np.float64, ctx)
        alg = mpsgb.DMRG2(maxdim=D, cutoff=1e-12, backend=mpsgb.GB300Backend(prec))
        psi, envs, eps, hist = mpsgb.find_groundstate(psi, H, alg, maxsweeps=6)
        # final energy evaluated with FP64 environments
        fenvs = mpsgb.FiniteEnvironments(psi, H)
        res[prec] = mpsgb.expectation_value(psi, H, fenvs, 0)
    assert abs(res["bf16x3"] - res["fp64"]) < 1e-7 * abs(res["fp64"]), res


def test_dmrg2_split_precision_gram_svd_vs_oracle(ctx):
    """The chosen form (bf16x3 contractions, Gram SVD, FP64 Lanczos) against the FP64
    oracle on the same seeded problem: relative energy error below 1e-9."""
    L_, D = 12, 64
    terms = M.heisenberg_terms(L_, dtype=np.float64)
    As = P.random_initial_tensors(L_, 2, D, 77, np.float64)
    oH = M.finite_mpo_hamiltonian(L_, 2, terms, dtype=np.float64)
    _, _, _, ohist = P.find_groundstate_dmrg2(P.finite_mps_from_tensors(As), oH,
                                              P.DMRG2(maxdim=D, cutoff=1e-12), maxsweeps=8)
    H = mpsgb.heisenberg_XXX(L_, dtype=np.float64)
    ctx.set_svd_method("gram")
    ctx.set_precision("bf16x3")
    try:
        psi = mpsgb.FiniteMPS.from_tensors(As, ctx)
        alg = mpsgb.DMRG2(maxdim=D, cutoff=1e-12, backend=mpsgb.GB300Backend("bf16x3"))
        psi, envs, eps, hist = mpsgb.find_groundstate(psi, H, alg, maxsweeps=8)
        fenvs = mpsgb.FiniteEnvironments(psi, H)
        e = mpsgb.expectation_value(psi, H, fenvs, 0)
    finally:
        ctx.set_svd_method("gesvd")
        ctx.set_precision("fp64")
    e_ref = ohist[-1][1]
    assert abs(e - e_ref) / abs(e_ref) < 1e-9, (e, e_ref)
