"""Two benchmark configurations run as written.

cfg 1 -- plain FP64 two-site DMRG, spin-1/2 Heisenberg chain, open, L = 32, ComplexF64,
seeded random initial MPS at D = 64, truncrank(64) & trunctol(atol = 1e-10), 10 sweeps
(src/algorithms/groundstate/dmrg.jl:211-354): the device energies per sweep against the
oracle's; then the split forms (tf32x3 / bf16x3 contractions, Gram factorisation, FP64
Lanczos) at the converged state against the same sweeps in FP64.

cfg 3 -- U(1) Heisenberg chain L = 100, total Sz = 0, D = 1024 (~20 charge sectors at the
central bond): at the central bond of the seeded state, the split-precision local solve
followed by its FP64 refinement (one FP64 matvec: Rayleigh quotient) against the plain FP64
solve from the same start vector and environments -- the metric's precision condition at
this configuration's contraction sizes (K up to ~1e5 in the AA-free nearest-neighbour
operator's IC/BE products)."""
import numpy as np
import pytest

import mpsgb
from mpsgb import u1 as HU
from mpsgb.operators import SPIN_HALF_CHARGES as QP
from oracle import models as M
from oracle import mps as P

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    return mpsgb.context(0)


def test_cfg1_dmrg2_heisenberg_L32_D64_complex(ctx, tmp_path):
    L_, D, sweeps = 32, 64, 10
    terms = M.heisenberg_terms(L_)
    As = P.random_initial_tensors(L_, 2, D, 1235, np.complex128)
    oH = M.finite_mpo_hamiltonian(L_, 2, terms)
    alg_o = P.DMRG2(maxdim=D, cutoff=1e-10)
    _, _, _, ohist = P.find_groundstate_dmrg2(P.finite_mps_from_tensors(As), oH, alg_o,
                                              maxsweeps=sweeps)
    H = mpsgb.heisenberg_XXX(L_)
    psi = mpsgb.FiniteMPS.from_tensors(As, ctx)
    psi, envs, eps, hist = mpsgb.find_groundstate(psi, H, mpsgb.DMRG2(maxdim=D, cutoff=1e-10),
                                                  maxsweeps=sweeps)
    assert len(hist) == len(ohist)
    for a, b in zip(hist, ohist):
        assert abs(a["energy"] - b[1]) <= 1e-10 * abs(b[1]), (a, b)
    # The split forms at the FP64 fixed point: from the converged state, sweeps with split
    # contractions and the Gram factorisation keep the energy (FP64 environments) of the
    # same sweeps in FP64.  (From the random start the runs are not comparable at 1e-9:
    # both stop once the Galerkin error meets the truncation error, ~1e-6 here, and their
    # truncated trajectories differ at that level.)
    path = str(tmp_path / "cfg1_state.npz")
    mpsgb.io.save_state(path, psi)

    def polish(prec, svd):
        ctx.set_svd_method(svd)
        ctx.set_precision(prec)
        try:
            p = mpsgb.io.load_state(path, ctx)
            alg = mpsgb.DMRG2(maxdim=D, cutoff=1e-10, backend=mpsgb.GB300Backend(prec))
            p, _, _, _ = mpsgb.find_groundstate(p, H, alg, maxsweeps=2)
        finally:
            ctx.set_svd_method("gesvd")
            ctx.set_precision("fp64")
        return mpsgb.expectation_value(p, H, mpsgb.FiniteEnvironments(p, H), 0)

    e64 = polish("fp64", "gesvd")
    # tf32x3 (22 significant bits per operand pair) holds it to 1e-9; bf16x3 (16 bits) to
    # ~1e-8 here (measured 1.0e-8): the energy error is quadratic in the operator's, and at
    # D = 64 every sweep re-truncates near small singular values
    for prec, bar in (("tf32x3", 1e-9), ("bf16x3", 3e-8)):
        e = polish(prec, "gram")
        assert abs(e - e64) <= bar * abs(e64), (prec, e, e64)


def test_cfg3_u1_L100_D1024_split_vs_fp64_at_the_central_bond(ctx):
    L_, D = 100, 1024
    pos = L_ // 2 - 1
    H = mpsgb.heisenberg_XXX(L_, dtype=np.float64, u1=True)
    As, qb = HU.random_u1_tensors(L_, D, 1237, 0, np.float64)
    psi = mpsgb.FiniteMPS.from_tensors(As, ctx, center=pos + 1, charges=(qb, QP))
    del As
    envs = mpsgb.FiniteEnvironments(psi, H, resident=False)
    x0 = mpsgb.ac2_from(psi.AL[pos], psi.ac(pos + 1))
    assert len(np.unique(x0.charges[0])) >= 15
    H64 = mpsgb.AC2_hamiltonian(pos, psi, H, envs, mpsgb.GB300Backend("fp64"))
    Hs = mpsgb.AC2_hamiltonian(pos, psi, H, envs, mpsgb.GB300Backend("bf16x3"))
    alg = lambda tol: mpsgb.Lanczos(krylovdim=30, maxiter=20, tol=tol, eager=False)
    l64, x64, i64 = mpsgb.fixedpoint(H64, x0, "SR", alg(1e-11))
    ls, xs, is_ = mpsgb.fixedpoint(Hs, x0, "SR", alg(1e-10))
    # the FP64 refinement step: Rayleigh quotient of the split solution with the FP64 operator
    y = H64(xs)
    e_s = y.dot(xs) / xs.dot(xs)
    y.axpy_(-e_s, xs)
    res_s = y.norm() / xs.norm()
    assert abs(e_s - l64) <= 1e-9 * abs(l64), (e_s, l64, ls)
    # the split operator alone is accurate only to its own rounding (first order)
    assert abs(ls - l64) <= 1e-5 * abs(l64)
    assert res_s < 1e-3
