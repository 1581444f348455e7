"""The host side of GradientGrassmann (mpsgb.optim: conjugate gradients with the Hager-Zhang
line search) driven by numpy points: a Rayleigh quotient on a Grassmann manifold, and the
finite-MPS energy through the oracle's fg / retract / transport (grassmann.jl:61-169),
converging to exact diagonalisation (gradient_grassmann.jl:80-121)."""
import numpy as np
import pytest

from mpsgb import optim
from oracle import grassmann as OG
from oracle import models as M
from oracle import mps as P


def _np_ops():
    add = lambda v, w, a, b: [a * x + b * y for x, y in zip(v, w)]
    scale = lambda v, a: [a * x for x in v]
    return add, scale


def test_cg_minimises_a_rayleigh_quotient():
    rng = np.random.default_rng(3)
    n, p = 30, 3
    A = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    A = A + A.conj().T
    W0, _ = np.linalg.qr(rng.standard_normal((n, p)) + 1j * rng.standard_normal((n, p)))
    sh = (n, 1, p)

    def fg(W):
        Wm = W[0].reshape(n, p, order="F")
        AW = A @ Wm
        G = AW - Wm @ (Wm.conj().T @ AW)
        return float(np.real(np.trace(Wm.conj().T @ AW))), [G.reshape(sh, order="F")]

    def retract(W, d, a):
        Wn, Zn = OG.retract_site(W[0], d[0], a)
        return [Wn], [Zn]

    def transport(v, W, d, a, Wn):
        return [OG.transport_site(v[0], W[0], d[0], a, Wn[0])]

    add, scale = _np_ops()
    alg = optim.ConjugateGradient(gradtol=1e-10, maxiter=500)
    W, f, g, nfg, hist = optim.optimize(fg, [W0.reshape(sh, order="F")], alg, retract,
                                        transport, lambda x, a, b: OG.inner(a, b), add, scale)
    assert hist[-1] <= 1e-10
    assert abs(f - np.sum(np.linalg.eigvalsh(A)[:p])) < 1e-10 * np.abs(A).max() * n
    Wm = W[0].reshape(n, p, order="F")
    assert np.abs(Wm.conj().T @ Wm - np.eye(p)).max() < 1e-12


def test_line_search_accepts_wolfe_points_only():
    # phi(c) = (c - 2)^2 along a straight line: the accepted step satisfies the Wolfe
    # conditions (sufficient decrease and the curvature condition)
    ls = optim.HagerZhangLineSearch()
    fg = lambda x: (float((x[0] - 2.0) ** 2), [np.array(2.0 * (x[0] - 2.0))])
    retract = lambda x, d, a: ([x[0] + a * d[0]], d)
    inner = lambda x, a, b: float(a[0] * b[0])
    x, f, g, xi, c, n = ls(fg, [np.array(0.0)], [np.array(1.0)], 4.0, [np.array(-4.0)], 0.1,
                           retract, inner)
    assert 0 < c and f - 4.0 <= 0.1 * c * -4.0 and g[0] * 1.0 >= 0.9 * -4.0 and n <= 10
    # from a step far beyond the minimiser the bracket and secant steps come back to it
    x, f, g, xi, c, n = ls(fg, [np.array(0.0)], [np.array(1.0)], 4.0, [np.array(-4.0)], 50.0,
                           retract, inner)
    assert f - 4.0 <= 0.1 * c * -4.0 and abs(g[0]) <= 0.9 * 4.0 and n <= 10


@pytest.mark.parametrize("L_,D,gx,bar", [(6, 4, 4.0, 1e-9), (10, 6, 1.0, 2e-9)])
def test_gradient_grassmann_reaches_ed_on_the_oracle(L_, D, gx, bar):
    # TFIM in its paramagnetic phase and at the critical point (where the bond matrices have
    # small singular values and the preconditioner amplifies rounding noise)
    terms = M.tfim_terms(L_, g=gx)
    H = M.finite_mpo_hamiltonian(L_, 2, terms)
    e_ed = M.ed_ground_energy(L_, 2, terms)[0]
    psi = P.finite_mps_from_tensors(P.random_initial_tensors(L_, 2, D, 17))
    # the point: the left-canonical form and the normalised last-bond factor
    AL, X = [], psi.C[0]
    for i in range(L_):
        A = np.einsum("ab,bsc->asc", X, psi.AR[i])
        Q, X = P.qr_pos(A.reshape(-1, A.shape[2], order="F"))
        AL.append(Q.reshape(A.shape[0], 2, Q.shape[1], order="F"))
    x0 = (AL, X / np.linalg.norm(X))
    add, scale = _np_ops()
    fg = lambda x: OG.fg(x[0], x[1], H)

    def retract(x, g, a):
        ALn, Cn, gn = OG.retract(x[0], x[1], g, a)
        return (ALn, Cn), gn

    transport = lambda h, x, g, a, xn: OG.transport(h, x[0], g, a, xn[0])
    precondition = lambda x, g: OG.precondition(x[0], x[1], g)
    alg = optim.ConjugateGradient(gradtol=1e-8, maxiter=300)
    x, f, g, nfg, hist = optim.optimize(fg, x0, alg, retract, transport,
                                        lambda x, a, b: OG.inner(a, b), add, scale,
                                        precondition)
    assert hist[-1] <= 1e-8, hist[-5:]
    assert -1e-12 * abs(e_ed) <= f - e_ed < bar * abs(e_ed), (f, e_ed)
    for A in x[0]:
        Q = A.reshape(-1, A.shape[2], order="F")
        assert np.abs(Q.conj().T @ Q - np.eye(Q.shape[1])).max() < 1e-13


def test_infinite_gradient_grassmann_on_the_oracle_reaches_the_closed_form():
    """One-site InfiniteMPS (grassmann.jl:109-122, 171-190): the restated optimiser with the
    oracle's fixed-point environments reaches the TFIM energy density of the closed form
    within the D = 4 truncation (paramagnetic g = 4, as the reference's infinite test)."""
    from oracle import vumps as V
    g = 4.0
    H = M.infinite_mpo_hamiltonian(1, 2, M.tfim_terms(1, g=g, periodic=True))
    rng = np.random.default_rng(2)
    A = rng.standard_normal((4, 2, 4)) + 1j * rng.standard_normal((4, 2, 4))
    psi = V.infinite_mps(A)
    add, scale = _np_ops()
    fg = lambda x: OG.fg_infinite(x, H[0], H.chans[0])
    transport = lambda h, x, gg, a, xn: [OG.transport_site(h[0], x.AL, gg[0], a, xn.AL)]
    x, f, gg, nfg, hist = optim.optimize(fg, psi, optim.ConjugateGradient(gradtol=1e-8,
                                                                          maxiter=200),
                                         OG.retract_infinite, transport,
                                         lambda x, a, b: OG.inner(a, b), add, scale,
                                         OG.precondition_infinite)
    assert hist[-1] <= 1e-8, hist[-5:]
    e_exact = M.tfim_infinite_energy_density(g)
    assert e_exact - 1e-12 <= f < e_exact + 1e-8, (f, e_exact)


def _cell_start(D, seed, n=2):
    from oracle import cell as Ce
    rng = np.random.default_rng(seed)
    As = [rng.standard_normal((D, 2, D)) + 1j * rng.standard_normal((D, 2, D)) for _ in range(n)]
    return Ce.infinite_mps(As)


def test_cell_gradient_is_the_derivative_of_the_cell_energy():
    """fg(::InfiniteMPS) with a two-site cell (grassmann.jl:171-190): along the geodesic of a
    direction d the energy of the cell changes at the rate inner(g, d)."""
    H = M.infinite_mpo_hamiltonian(2, 2, M.tfim_terms(2, g=0.8, periodic=True))
    psi = _cell_start(4, 5)
    f0, g0 = OG.fg_cell(psi, H)
    d = [-x for x in OG.precondition_cell(psi, g0)]
    slope = OG.inner(g0, d)
    assert slope < 0
    h = 1e-4
    fp = OG.fg_cell(OG.retract_cell(psi, d, h)[0], H)[0]
    fm = OG.fg_cell(OG.retract_cell(psi, d, -h)[0], H)[0]
    assert abs((fp - fm) / (2 * h) - slope) <= 1e-5 * abs(slope)


def test_cell_gradient_grassmann_on_the_oracle_reaches_the_closed_form():
    """GradientGrassmann on a two-site InfiniteMPS cell: the restated optimiser reaches the
    TFIM energy per site of the closed form within the D = 4 truncation."""
    g = 4.0
    H = M.infinite_mpo_hamiltonian(2, 2, M.tfim_terms(2, g=g, periodic=True))
    add, scale = _np_ops()
    x, f, gg, nfg, hist = optim.optimize(lambda x: OG.fg_cell(x, H), _cell_start(4, 2),
                                         optim.ConjugateGradient(gradtol=1e-8, maxiter=300),
                                         OG.retract_cell, OG.transport_cell,
                                         lambda x, a, b: OG.inner(a, b), add, scale,
                                         OG.precondition_cell)
    assert hist[-1] <= 1e-8, hist[-5:]
    e_exact = M.tfim_infinite_energy_density(g)
    assert e_exact - 1e-12 <= f / 2 < e_exact + 1e-8, (f / 2, e_exact)


def test_cell_idmrg_on_the_oracle():
    """IDMRG (one-site updates) on InfiniteMPS cells (idmrg.jl:85-229): on a one-site cell the
    cell restatement repeats the one-site oracle step for step, and on a two-site TFIM cell it
    reaches the VUMPS energy per site of the same bond dimension."""
    from oracle import cell as Ce
    from oracle import vumps as V
    g = 0.9
    rng = np.random.default_rng(4)
    A = rng.standard_normal((6, 2, 6)) + 1j * rng.standard_normal((6, 2, 6))
    H1 = M.infinite_mpo_hamiltonian(1, 2, M.tfim_terms(1, g=g, periodic=True))
    _, _, _, e1, h1 = V.idmrg(V.infinite_mps(A), H1, tol=1e-9, maxiter=40)
    _, _, _, ec, hc = Ce.idmrg1(Ce.infinite_mps([A]), H1, tol=1e-9, maxiter=40)
    assert len(h1) == len(hc)
    for a, b in zip(h1, hc):
        assert abs(a[2] - b[2]) <= 1e-8 * max(1.0, a[2]) and abs(np.real(a[1]) - b[1]) < 1e-10
    H2 = M.infinite_mpo_hamiltonian(2, 2, M.tfim_terms(2, g=g, periodic=True))
    As = [rng.standard_normal((6, 2, 6)) + 1j * rng.standard_normal((6, 2, 6)) for _ in range(2)]
    psi, GL, GR, eps, hist = Ce.idmrg1(Ce.infinite_mps(As), H2, tol=1e-9, maxiter=200)
    assert eps <= 1e-9
    vpsi, vGL, vGR, veps, vhist = Ce.vumps(Ce.infinite_mps(As), H2, tol=1e-10, maxiter=100)
    assert abs(Ce.energy(psi, H2, GL, GR) - Ce.energy(vpsi, H2, vGL, vGR)) / 2 < 1e-8


def test_cell_tdvp_on_the_oracle():
    """TDVP on InfiniteMPS cells (tdvp.jl:72-133): the cell restatement on a one-site cell
    repeats the one-site oracle step, a real-time step of a two-site ground state keeps its
    energy, and an imaginary-time step lowers the energy of a random state."""
    from oracle import cell as Ce
    from oracle import vumps as V
    rng = np.random.default_rng(6)
    A = rng.standard_normal((4, 2, 4)) + 1j * rng.standard_normal((4, 2, 4))
    H1 = M.infinite_mpo_hamiltonian(1, 2, M.tfim_terms(1, g=0.7, periodic=True))
    p1, _, _ = V.tdvp_timestep_infinite(V.infinite_mps(A), H1, 0.05)
    pc, _, _ = Ce.tdvp_timestep(Ce.infinite_mps([A]), H1, 0.05)
    assert np.abs(p1.AL - pc.AL[0]).max() < 1e-10 and np.abs(p1.C - pc.C[0]).max() < 1e-10
    H2 = M.infinite_mpo_hamiltonian(2, 2, M.tfim_terms(2, g=0.7, periodic=True))
    As = [rng.standard_normal((6, 2, 6)) + 1j * rng.standard_normal((6, 2, 6)) for _ in range(2)]
    gs, GL, GR, _, _ = Ce.vumps(Ce.infinite_mps(As), H2, tol=1e-10, maxiter=100)
    e0 = Ce.energy(gs, H2, GL, GR)
    p2, GL2, GR2 = Ce.tdvp_timestep(gs, H2, 0.1, GL, GR)
    assert abs(Ce.energy(p2, H2, GL2, GR2) - e0) < 1e-8
    psi = Ce.infinite_mps(As)
    GL, GR = Ce.infinite_envs(psi, H2)
    p3, GL3, GR3 = Ce.tdvp_timestep(psi, H2, 0.1, GL, GR, imaginary=True)
    assert Ce.energy(p3, H2, GL3, GR3) < Ce.energy(psi, H2, GL, GR)
