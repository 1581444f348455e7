"""GradientGrassmann on the device (src/algorithms/grassmann.jl, gradient_grassmann.jl)
against the oracle: fg, precondition, retract and transport at the same point and direction,
then whole optimisations reaching exact diagonalisation, as the reference's groundstate test
(test/algorithms/groundstate.jl:177-192: TFIM g = 4, L = 10, D = 6)."""
import numpy as np
import pytest

import mpsgb
from mpsgb import grassmann as G
from oracle import grassmann as OG
from oracle import models as M
from oracle import mps as P

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    return mpsgb.context(0)


def _point(L_, D, seed):
    psi = P.finite_mps_from_tensors(P.random_initial_tensors(L_, 2, D, seed))
    AL, X = [], psi.C[0]
    for i in range(L_):
        A = np.einsum("ab,bsc->asc", X, psi.AR[i])
        Q, X = P.qr_pos(A.reshape(-1, A.shape[2], order="F"))
        AL.append(Q.reshape(A.shape[0], 2, Q.shape[1], order="F"))
    return AL, X / np.linalg.norm(X)


def _dev_point(ctx, AL, C):
    T = lambda k, a: mpsgb.DeviceTensor.from_numpy(ctx, k, a)
    return G.GrassmannPoint([T("mps", a) for a in AL], T("bond", C))


def _dev_tangent(x, Z):
    return [G.GrassmannTangent(x.AL[i], mpsgb.DeviceTensor.from_numpy(x.psi.ctx, "mps", z))
            for i, z in enumerate(Z)]


def _nontrivial(AL):
    # sites whose tangent space is not empty (Dl d > Dr)
    return [i for i, a in enumerate(AL) if a.shape[0] * a.shape[1] > a.shape[2]]


def test_grassmann_steps_match_the_oracle(ctx):
    L_, D = 8, 6
    H = M.finite_mpo_hamiltonian(L_, 2, M.tfim_terms(L_, g=1.0))
    Hd = mpsgb.transverse_field_ising(L_, g=1.0)
    AL, C = _point(L_, D, 71)
    x = _dev_point(ctx, AL, C)
    envs = mpsgb.FiniteEnvironments(x.psi, Hd, ctx)
    # fg
    f_o, g_o = OG.fg(AL, C, H)
    f_d, g_d = G.fg(x, Hd, envs)
    assert abs(f_d - f_o) <= 1e-12 * abs(f_o)
    gmax = max(np.linalg.norm(z) for z in g_o)
    for i in range(L_):
        assert np.linalg.norm(g_d[i].Z.numpy() - g_o[i]) <= 1e-12 * gmax, i
    assert abs(G.inner(x, g_d, g_d) - OG.inner(g_o, g_o)) <= 1e-12 * OG.inner(g_o, g_o)
    # precondition (the sites with an empty tangent space carry amplified rounding noise)
    Pg_o = OG.precondition(AL, C, g_o)
    Pg_d = G.precondition(x, _dev_tangent(x, g_o))
    nt = _nontrivial(AL)
    pmax = max(np.linalg.norm(Pg_o[i]) for i in nt)
    for i in nt:
        assert np.linalg.norm(Pg_d[i].Z.numpy() - Pg_o[i]) <= 1e-11 * pmax, i
    # retract and transport along the same direction
    d = [-z if i in nt else np.zeros_like(z) for i, z in enumerate(Pg_o)]
    a = 0.37
    ALn_o, Cn_o, xi_o = OG.retract(AL, C, d, a)
    xn, xi_d = G.retract(x, _dev_tangent(x, d), a)
    for i in range(L_):
        assert np.abs(xn.AL[i].numpy() - ALn_o[i]).max() <= 1e-12, i
        assert np.abs(xi_d[i].Z.numpy() - xi_o[i]).max() <= 1e-12 * max(1.0, pmax), i
    h_o = OG.transport(g_o, AL, d, a, ALn_o)
    h_d = G.transport(_dev_tangent(x, g_o), x, _dev_tangent(x, d), a, xn)
    for i in range(L_):
        assert np.abs(h_d[i].Z.numpy() - h_o[i]).max() <= 1e-12 * gmax, i
    # transport is an isometry of the tangent spaces
    n0, n1 = OG.inner(g_o, g_o), G.inner(xn, h_d, h_d)
    assert abs(n1 - n0) <= 1e-10 * n0


@pytest.mark.parametrize("gx,bar", [(4.0, 1e-9), (1.0, 2e-9)])
def test_gradient_grassmann_reaches_ed(ctx, gx, bar):
    L_, D = 10, 6
    terms = M.tfim_terms(L_, g=gx)
    e_ed = M.ed_ground_energy(L_, 2, terms)[0]
    psi = mpsgb.FiniteMPS.from_tensors(P.random_initial_tensors(L_, 2, D, 5), ctx)
    alg = mpsgb.GradientGrassmann(tol=1e-8, maxiter=300)
    out, envs, normgrad, hist = mpsgb.find_groundstate(psi, mpsgb.transverse_field_ising(L_, g=gx),
                                                       alg)
    assert normgrad <= 1e-8, hist["normgrad"][-5:]
    e = mpsgb.expectation_value(out, mpsgb.transverse_field_ising(L_, g=gx), envs)
    assert abs(e - hist["energy"]) <= 1e-10 * abs(e)
    assert -1e-12 * abs(e_ed) <= e - e_ed < bar * abs(e_ed), (e, e_ed)
    for A in out.AR:
        a = A.numpy()
        Q = a.reshape(a.shape[0], -1, order="F")
        assert np.abs(Q @ Q.conj().T - np.eye(Q.shape[0])).max() < 1e-12


def _A(D, seed):
    rng = np.random.default_rng(seed)
    return rng.standard_normal((D, 2, D)) + 1j * rng.standard_normal((D, 2, D))


def test_infinite_gradient_is_the_derivative_of_the_energy(ctx):
    """fg(::InfiniteMPS) (grassmann.jl:171-190): along the geodesic of a direction d the
    energy density changes at the rate inner(g, d) (central differences)."""
    H = mpsgb.transverse_field_ising(1, g=0.8, infinite=True)
    psi = mpsgb.InfiniteMPS.from_tensor(_A(8, 4), ctx)
    envs = mpsgb.InfiniteEnvironments(psi, H)
    f0, g0 = G.fg_infinite(psi, H, envs)
    d = G.scale(G.precondition_infinite(psi, g0), -1.0)
    slope = G.inner(psi, g0, d)
    assert slope < 0
    h = 1e-4
    fp = G.fg_infinite(G.retract_infinite(psi, d, h)[0], H, envs)[0]
    fm = G.fg_infinite(G.retract_infinite(psi, d, -h)[0], H, envs)[0]
    assert abs((fp - fm) / (2 * h) - slope) <= 1e-5 * abs(slope)


@pytest.mark.parametrize("gx,D", [(4.0, 6), (0.8, 10)])
def test_infinite_gradient_grassmann_matches_vumps(ctx, gx, D):
    """GradientGrassmann on a one-site InfiniteMPS (the reference's infinite groundstate
    test, test/algorithms/groundstate.jl:268-292) reaches the VUMPS fixed point of the same
    bond dimension and the TFIM closed form within the truncation."""
    H = mpsgb.transverse_field_ising(1, g=gx, infinite=True)
    psi = mpsgb.InfiniteMPS.from_tensor(_A(D, 1), ctx)
    alg = mpsgb.GradientGrassmann(tol=1e-8, maxiter=300)
    out, envs, normgrad, hist = mpsgb.find_groundstate(psi, H, alg)
    assert normgrad <= 1e-8, hist["normgrad"][-5:]
    e = mpsgb.infinite.energy_density(out, envs)
    vpsi = mpsgb.InfiniteMPS.from_tensor(_A(D, 1), ctx)
    vpsi, venvs, eps, vhist = mpsgb.find_groundstate_vumps(vpsi, H, mpsgb.VUMPS(tol=1e-10,
                                                                                maxiter=200))
    e_exact = M.tfim_infinite_energy_density(gx)
    assert e >= e_exact - 1e-10
    assert abs(e - vhist[-1]["energy"]) <= 1e-9 * abs(e), (e, vhist[-1]["energy"])
    assert mpsgb.infinite.galerkin(out, envs) < 1e-6


def _cell_As(D, seed, n=2):
    rng = np.random.default_rng(seed)
    return [rng.standard_normal((D, 2, D)) + 1j * rng.standard_normal((D, 2, D))
            for _ in range(n)]


def _relerr(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def test_cell_fg_precondition_and_retract_match_the_oracle(ctx):
    """GradientGrassmann's pieces on a two-site InfiniteMPS cell (grassmann.jl:85-122,
    171-190) against the oracle's cell restatement at the same point: the cell energy, the
    per-site gradients, the preconditioned direction and the retracted point."""
    from mpsgb import cell as GC
    from oracle import cell as Ce
    As = _cell_As(6, 5)
    H = mpsgb.transverse_field_ising(2, g=0.8, infinite=True)
    oH = M.infinite_mpo_hamiltonian(2, 2, M.tfim_terms(2, g=0.8, periodic=True))
    opsi = Ce.infinite_mps(As)
    psi = GC.InfiniteMPSCell.from_tensors(As, ctx)
    envs = GC.InfiniteEnvironmentsCell(psi, H)
    f, g = G.fg_cell(psi, H, envs)
    of, og = OG.fg_cell(opsi, oH)
    assert abs(f - of) <= 1e-9 * abs(of), (f, of)
    p, op = G.precondition_cell(psi, g), OG.precondition_cell(opsi, og)
    for s in range(2):
        assert _relerr(g[s].Z.numpy(), og[s]) <= 1e-6, s
        assert _relerr(p[s].Z.numpy(), op[s]) <= 1e-5, s
    xn, _ = G.retract_cell(psi, G.scale(p, -1.0), 0.05)
    oxn, _ = OG.retract_cell(opsi, [-x for x in op], 0.05)
    for s in range(2):
        assert _relerr(xn.AL[s].numpy(), oxn.AL[s]) <= 1e-6, s
        assert _relerr(xn.C[s].numpy(), oxn.C[s]) <= 1e-6, s


def test_cell_gradient_grassmann_reaches_the_closed_form(ctx):
    """GradientGrassmann on a two-site InfiniteMPS cell (TFIM g = 4, D = 4): the gradient
    vanishes, the energy per site is the closed form within the truncation, and the state is
    a VUMPS fixed point (Galerkin error)."""
    from mpsgb import cell as GC
    H = mpsgb.transverse_field_ising(2, g=4.0, infinite=True)
    psi = GC.InfiniteMPSCell.from_tensors(_cell_As(4, 2), ctx)
    out, envs, normgrad, hist = mpsgb.find_groundstate(
        psi, H, mpsgb.GradientGrassmann(tol=1e-8, maxiter=300))
    assert normgrad <= 1e-8, hist["normgrad"][-5:]
    e_exact = M.tfim_infinite_energy_density(4.0)
    assert e_exact - 1e-12 <= hist["energy"] < e_exact + 1e-8, (hist["energy"], e_exact)
    assert GC.galerkin(out, envs) < 1e-6
