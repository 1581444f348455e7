"""CPU tests of the oracle: pinned by the reference's known answers, by exact
diagonalisation built from the lattice terms, and by closed forms."""
import json
import os

import numpy as np
import pytest

from oracle import derivatives as dv
from oracle import krylov as K
from oracle import models as M
from oracle import mps as P

HERE = os.path.dirname(os.path.abspath(__file__))
KAT = json.load(open(os.path.join(HERE, "golden", "known_answers.json")))


def test_tfim_doctest_known_answer():
    """find_groundstate.jl:49-64: DMRG2 from the all-ones product state, truncrank(16)."""
    L = 4
    H = M.finite_mpo_hamiltonian(L, 2, M.tfim_doctest_terms(L), dtype=np.float64)
    psi = P.finite_mps_from_tensors([np.ones((1, 2, 1)) for _ in range(L)])
    _, _, _, hist = P.find_groundstate_dmrg2(psi, H, P.DMRG2(maxdim=16), maxsweeps=30)
    kat = KAT["tfim_L4_doctest"]
    assert round(hist[-1][1], 4) == kat["energy_rounded_4"]


def test_heisenberg_L20_known_answer():
    """test/algorithms/groundstate.jl:151-175: E = -8.6824724 for L = 20, spin 1/2."""
    L = 20
    H = M.finite_mpo_hamiltonian(L, 2, M.heisenberg_terms(L, dtype=np.float64), dtype=np.float64)
    psi = P.finite_mps_from_tensors(P.random_initial_tensors(L, 2, 8, 5, np.float64))
    _, _, _, hist = P.find_groundstate_dmrg2(psi, H, P.DMRG2(maxdim=48, cutoff=1e-12), maxsweeps=12)
    kat = KAT["heisenberg_L20_spin_half"]
    assert abs(hist[-1][1] - kat["energy"]) < kat["atol"]


@pytest.mark.parametrize("L", [6, 9])
def test_dmrg2_matches_ed(L):
    terms = M.xxz_terms(L, Jxy=1.0, Jz=1.5, hz=0.3)
    H = M.finite_mpo_hamiltonian(L, 2, terms)
    psi = P.finite_mps_from_tensors(P.random_initial_tensors(L, 2, 8, L))
    _, _, _, hist = P.find_groundstate_dmrg2(psi, H, P.DMRG2(maxdim=64), maxsweeps=20)
    e = M.ed_ground_energy(L, 2, terms)[0]
    assert abs(hist[-1][1] - e) < 1e-9


def test_tfim_free_fermion_closed_form():
    L = 10
    terms = M.tfim_terms(L, g=0.8)
    e_ff = M.tfim_open_chain_energy(L, g=0.8)
    e_ed = M.ed_ground_energy(L, 2, terms)[0]
    assert abs(e_ff - e_ed) < 1e-10


def test_golden_ed_fixture():
    e = float(np.load(os.path.join(HERE, "golden", "ed_heisenberg_L10.npz"))["energy"])
    assert abs(e - M.ed_ground_energy(10, 2, M.heisenberg_terms(10))[0]) < 1e-12


@pytest.mark.parametrize("name", ["ac2_heisenberg_c128", "ac2_tfim_edge_f64", "ac2_j1j2_f64"])
def test_golden_ac2_fixtures_reproduce(name):
    f = np.load(os.path.join(HERE, "golden", f"{name}.npz"))
    op = dv.JordanAC2(f["GL"], f["W1"], f["W2"], f["GR"])
    y = op(f["x"])
    assert np.allclose(y, f["y"], rtol=0, atol=1e-12 * np.abs(f["y"]).max())
    assert ",".join(op.terms()) == str(f["terms"])


@pytest.mark.parametrize("model", ["heis", "tfim", "j1j2", "xxz_field"])
def test_jordan_ac2_equals_generic_mpo_contraction(model):
    """The Jordan decomposition + prepare folds are the same linear map as the generic
    MPO_AC2 contraction (mpo_derivatives.jl:144-153)."""
    if model == "heis":
        L, terms, dt = 8, M.heisenberg_terms(8), np.complex128
    elif model == "tfim":
        L, terms, dt = 8, M.tfim_terms(8, g=1.3, dtype=np.float64), np.float64
    elif model == "xxz_field":
        L, terms, dt = 8, M.xxz_terms(8, 1.0, 0.7, 0.4), np.complex128
    else:
        L, terms, dt = 12, M.j1j2_cylinder_terms(4, 3), np.float64
    H = M.finite_mpo_hamiltonian(L, 2, terms, dtype=dt)
    psi = P.finite_mps_from_tensors(P.random_initial_tensors(L, 2, 6, 3, dt))
    envs = P.FiniteEnvironments(psi, H)
    rng = np.random.default_rng(0)
    for pos in (0, L // 2 - 1, L - 2):
        GL, GR = envs.leftenv(pos, psi), envs.rightenv(pos + 1, psi)
        x = rng.standard_normal((GL.shape[0], 2, GR.shape[0], 2)).astype(dt)
        y1 = dv.JordanAC2(GL, H[pos], H[pos + 1], GR)(x)
        y2 = dv.JordanAC2(GL, H[pos], H[pos + 1], GR, prepare=False)(x)
        y3 = dv.mpo_ac2_apply(GL, H[pos], H[pos + 1], GR, x)
        assert np.allclose(y1, y3, atol=1e-11 * np.abs(y3).max())
        assert np.allclose(y2, y3, atol=1e-11 * np.abs(y3).max())


def test_jordan_ac_equals_generic():
    L = 8
    H = M.finite_mpo_hamiltonian(L, 2, M.xxz_terms(L, 1.0, 0.6, 0.2))
    psi = P.finite_mps_from_tensors(P.random_initial_tensors(L, 2, 6, 4))
    envs = P.FiniteEnvironments(psi, H)
    rng = np.random.default_rng(2)
    for pos in (0, 3, L - 1):
        GL, GR = envs.leftenv(pos, psi), envs.rightenv(pos, psi)
        x = rng.standard_normal((GL.shape[0], 2, GR.shape[0])) + 0j
        y1 = dv.JordanAC(GL, H[pos], GR)(x)
        y2 = dv.mpo_ac_apply(GL, H[pos], GR, x)
        assert np.allclose(y1, y2, atol=1e-12 * np.abs(y2).max())


def test_linearity_of_ac2_in_the_hamiltonian():
    """AC2_hamiltonian(H1 + H2) x == AC2(H1) x + AC2(H2) x at fixed environments of each
    (the LazySum linearity property of test/operators/lazysum.jl:79-260) -- checked here
    through the energy functional: <psi|H1+H2|psi> = <H1> + <H2>."""
    L = 8
    t1 = M.heisenberg_terms(L)
    t2 = [((i,), 0.3 * M.spin_ops()[2]) for i in range(L)]
    psi = P.finite_mps_from_tensors(P.random_initial_tensors(L, 2, 6, 9))
    e = []
    for terms in (t1, t2, t1 + t2):
        H = M.finite_mpo_hamiltonian(L, 2, terms)
        envs = P.FiniteEnvironments(psi, H)
        e.append(P.expectation_value(psi, H, envs, 0))
    assert abs(e[0] + e[1] - e[2]) < 1e-12


def test_lanczos_restart_matches_dense():
    rng = np.random.default_rng(3)
    A = rng.standard_normal((200, 200))
    A = A + A.T
    x0 = rng.standard_normal(200)
    val, vec, info = K.lanczos_eigsolve(lambda v: A @ v, x0, krylovdim=20, maxiter=200, tol=1e-10)
    assert abs(val - np.linalg.eigvalsh(A)[0]) < 1e-8
    assert info.numiter > 1


def test_exponentiate_matches_expm():
    import scipy.linalg as sl
    rng = np.random.default_rng(4)
    A = rng.standard_normal((60, 60))
    A = (A + A.T) / 10
    x0 = rng.standard_normal(60) + 0j
    y, info = K.lanczos_exponentiate(lambda v: A @ v, -0.7j, x0, krylovdim=20, tol=1e-12)
    assert np.allclose(y, sl.expm(-0.7j * A) @ x0, atol=1e-10)


def test_transfer_environment_energy_consistency():
    """GL/GR built by transfer_left/right give the same energy at every site."""
    L = 8
    H = M.finite_mpo_hamiltonian(L, 2, M.heisenberg_terms(L))
    psi = P.finite_mps_from_tensors(P.random_initial_tensors(L, 2, 6, 8))
    envs = P.FiniteEnvironments(psi, H)
    e0 = P.expectation_value(psi, H, envs, 0)
    # move the centre right with positive QR and evaluate again
    for i in range(L - 1):
        ac = psi.ac(i)
        Dl, d, Dr = ac.shape
        Q, R = P.qr_pos(ac.reshape(Dl * d, Dr, order="F"))
        psi.AL[i] = Q.reshape(Dl, d, -1, order="F")
        psi.C[i + 1] = R
        psi.center = i + 1
        ei = P.expectation_value(psi, H, envs, i + 1)
        assert abs(ei - e0) < 1e-11


def test_oracle_vumps_tfim_closed_form():
    """VUMPS on the infinite TFIM (g = 0.5) reaches the free-fermion energy density."""
    from oracle import vumps as V
    H = M.infinite_mpo_hamiltonian(1, 2, M.tfim_terms(1, g=0.5, periodic=True))
    rng = np.random.default_rng(1)
    A = rng.standard_normal((12, 2, 12)) + 1j * rng.standard_normal((12, 2, 12))
    psi, GL, GR, eps, hist = V.vumps(V.infinite_mps(A), H, tol=1e-10, maxiter=100)
    assert eps <= 1e-10
    assert abs(hist[-1][1] - M.tfim_infinite_energy_density(0.5)) < 1e-12


def test_oracle_infinite_tdvp_imaginary_and_real_time():
    """One-site infinite TDVP (tdvp.jl:91-133): imaginary time reaches the TFIM closed form,
    real time conserves the energy density."""
    from oracle import vumps as V
    g = 0.5
    oH = M.infinite_mpo_hamiltonian(1, 2, M.tfim_terms(1, g=g, periodic=True))
    rng = np.random.default_rng(6)
    A = rng.standard_normal((8, 2, 8)) + 1j * rng.standard_normal((8, 2, 8))
    psi = V.infinite_mps(A)
    GL = GR = None
    for _ in range(60):
        psi, GL, GR = V.tdvp_timestep_infinite(psi, oH, 0.2, GL, GR, imaginary=True)
    e0 = V.energy_density(psi, oH[0], GL, GR)
    assert abs(e0 - M.tfim_infinite_energy_density(g)) < 1e-10
    # quench to g = 0.8 and evolve in real time: the energy density is conserved
    oH2 = M.infinite_mpo_hamiltonian(1, 2, M.tfim_terms(1, g=0.8, periodic=True))
    GL, GR = V.infinite_envs(psi, oH2[0], oH2.chans[0])
    e1 = V.energy_density(psi, oH2[0], GL, GR)
    for _ in range(5):
        psi, GL, GR = V.tdvp_timestep_infinite(psi, oH2, 0.05, GL, GR)
    assert abs(V.energy_density(psi, oH2[0], GL, GR) - e1) < 1e-6


def test_rotated_xxz_is_unitarily_equivalent():
    """The sublattice rotation (pi about x on every other site) maps the XXZ bond term
    Jxy (SxSx + SySy) + Jz SzSz onto Jxy (SxSx - SySy) - Jz SzSz: same spectrum, and the
    open-chain ground energies agree (ED, L = 8)."""
    sx, sy, sz = M.spin_ops()
    h = (M.two_site(sx, sx) + M.two_site(sy, sy) + 1.5 * M.two_site(sz, sz)).reshape(4, 4)
    hr = (M.two_site(sx, sx) - M.two_site(sy, sy) - 1.5 * M.two_site(sz, sz)).reshape(4, 4)
    U = np.kron(np.eye(2), 2 * sx)
    assert np.allclose(U @ h @ U.conj().T, hr, atol=1e-15)
    e = M.ed_ground_energy(8, 2, M.xxz_terms(8, 1.0, 1.5))[0]
    er = M.ed_ground_energy(8, 2, M.xxz_terms(8, 1.0, 1.5, rotated=True))[0]
    assert abs(e - er) < 1e-12


def test_oracle_vumps_rotated_xxz_bethe_ansatz():
    """One-site VUMPS on the rotated XXZ chain in the Neel phase (Delta = 3) approaches the
    Bethe-ansatz energy density from above (variational, D = 12)."""
    from oracle import vumps as V
    delta = 3.0
    H = M.infinite_mpo_hamiltonian(1, 2, M.xxz_terms(1, 1.0, delta, periodic=True,
                                                     rotated=True))
    rng = np.random.default_rng(7)
    A = rng.standard_normal((12, 2, 12)) + 1j * rng.standard_normal((12, 2, 12))
    psi, GL, GR, eps, hist = V.vumps(V.infinite_mps(A), H, tol=1e-10, maxiter=40)
    de = hist[-1][1] - M.xxz_infinite_energy_density(delta)
    assert 0.0 <= de < 2e-8
    # the closed form at Delta = 1 is 1/4 - ln 2, and it is continuous there
    assert abs(M.xxz_infinite_energy_density(1.0 + 1e-9) - (0.25 - np.log(2.0))) < 1e-6


def test_oracle_idmrg_tfim_closed_form():
    """One-site IDMRG (idmrg.jl:194-228) on the infinite TFIM (g = 0.5) reaches the
    free-fermion energy density, and its last energy change per site agrees with it."""
    from oracle import vumps as V
    H = M.infinite_mpo_hamiltonian(1, 2, M.tfim_terms(1, g=0.5, periodic=True))
    rng = np.random.default_rng(1)
    A = rng.standard_normal((12, 2, 12)) + 1j * rng.standard_normal((12, 2, 12))
    psi, GL, GR, eps, hist = V.idmrg(V.infinite_mps(A), H, tol=1e-10, maxiter=100)
    exact = M.tfim_infinite_energy_density(0.5)
    assert eps <= 1e-10
    assert abs(V.energy_density(psi, H[0], GL, GR) - exact) < 1e-12
    assert abs(hist[-1][1] - exact) < 1e-10


def test_oracle_cell_of_one_site_equals_one_site_vumps():
    """The unit-cell restatement (oracle/cell.py) with L = 1 takes the one-site VUMPS path
    step for step: same iterations, energies and tensors."""
    from oracle import cell as Ce
    from oracle import vumps as V
    H = M.infinite_mpo_hamiltonian(1, 2, M.tfim_terms(1, g=0.5, periodic=True))
    rng = np.random.default_rng(1)
    A = rng.standard_normal((12, 2, 12)) + 1j * rng.standard_normal((12, 2, 12))
    p1, _, _, e1, h1 = V.vumps(V.infinite_mps(A), H, tol=1e-10, maxiter=100)
    pc, _, _, ec, hc = Ce.vumps(Ce.infinite_mps([A]), H, tol=1e-10, maxiter=100)
    assert len(h1) == len(hc)
    assert abs(h1[-1][1] - hc[-1][1]) < 1e-13
    assert np.allclose(p1.AL, pc.AL[0], atol=1e-12)


def test_oracle_two_site_cell_vumps():
    """VUMPS on a two-site cell: the TFIM reaches the free-fermion energy density, and the
    Neel-ordered XXZ chain (Delta = 3, no sublattice rotation) approaches the Bethe ansatz
    from above."""
    from oracle import cell as Ce
    rng = np.random.default_rng(3)
    H = M.infinite_mpo_hamiltonian(2, 2, M.tfim_terms(2, g=0.5, periodic=True))
    As = [rng.standard_normal((10, 2, 10)) + 1j * rng.standard_normal((10, 2, 10))
          for _ in range(2)]
    _, _, _, eps, hist = Ce.vumps(Ce.infinite_mps(As), H, tol=1e-10, maxiter=100)
    assert eps <= 1e-10
    assert abs(hist[-1][1] - M.tfim_infinite_energy_density(0.5)) < 1e-12
    Hx = M.infinite_mpo_hamiltonian(2, 2, M.xxz_terms(2, 1.0, 3.0, periodic=True))
    As = [rng.standard_normal((12, 2, 12)) + 1j * rng.standard_normal((12, 2, 12))
          for _ in range(2)]
    _, _, _, _, hist = Ce.vumps(Ce.infinite_mps(As), Hx, tol=1e-10, maxiter=30)
    de = hist[-1][1] - M.xxz_infinite_energy_density(3.0)
    assert 0.0 <= de < 2e-8


def test_oracle_idmrg2_tfim():
    """IDMRG2 (idmrg.jl:230-338) on a two-site cell grows the bond from D = 4 under
    truncrank(16) and reaches the TFIM energy density; its energy change per cycle is the
    energy of one unit cell."""
    from oracle import cell as Ce
    rng = np.random.default_rng(3)
    H = M.infinite_mpo_hamiltonian(2, 2, M.tfim_terms(2, g=0.5, periodic=True))
    As = [rng.standard_normal((4, 2, 4)) + 1j * rng.standard_normal((4, 2, 4))
          for _ in range(2)]
    psi, GL, GR, eps, hist = Ce.idmrg2(Ce.infinite_mps(As), H, maxdim=16, atol=1e-12,
                                       tol=1e-10, maxiter=100)
    exact = M.tfim_infinite_energy_density(0.5)
    assert eps <= 1e-10
    assert psi.AL[0].shape[0] > 4
    assert abs(Ce.energy(psi, H, GL, GR) / 2 - exact) < 1e-10
    assert abs(hist[-1][1] - 2 * exact) < 1e-8
    with pytest.raises(ValueError):
        Ce.idmrg2(Ce.infinite_mps(As[:1]), M.infinite_mpo_hamiltonian(
            1, 2, M.tfim_terms(1, g=0.5, periodic=True)), maxdim=8)


def test_oracle_dmrg3s_escapes_a_small_bond():
    """Single-site DMRG cannot grow the bond of a D = 2 start and stalls far above the ground
    state; with the DMRG3S gauge (post_expand/dmrg3s.jl:155-221, noise 0.1, decay 0.8,
    truncrank(16)) the perturbation opens new directions and the energy reaches exact
    diagonalisation -- the mechanism of the reference's 'DMRG3S escapes local minimum' test
    (test/algorithms/groundstate.jl:151-175)."""
    L_ = 10
    H = M.finite_mpo_hamiltonian(L_, 2, M.heisenberg_terms(L_))
    e_ed = M.ed_ground_energy(L_, 2, M.heisenberg_terms(L_))[0]
    psi0 = P.finite_mps_from_tensors(P.random_initial_tensors(L_, 2, 2, 5))
    _, _, _, h_plain = P.find_groundstate_dmrg(psi0, H, P.DMRG(tol=1e-10, maxiter=12))
    alg = P.DMRG(tol=1e-10, maxiter=12, alg_gauge=P.DMRG3S(0.1, 0.8, 16, 1e-12))
    _, _, _, h_3s = P.find_groundstate_dmrg(psi0, H, alg)
    assert h_plain[-1][1] - e_ed > 0.1
    assert 0.0 <= h_3s[-1][1] - e_ed < 1e-7


def _mps_vector(psi):
    """The state vector of a small finite MPS with its centre bond at psi.center."""
    c = psi.center
    ts = [psi.AL[i] for i in range(c)] + [psi.AC(c)] + [psi.AR[i] for i in range(c + 1, len(psi))]
    v = ts[0]
    for t in ts[1:]:
        v = np.tensordot(v, t, axes=([v.ndim - 1], [0]))
    return v.reshape(-1)


def test_oracle_optimal_expand_preserves_the_state_and_reaches_ed():
    """OptimalExpand (changebonds/optimalexpand.jl:122-187) adds directions with zero
    weight: one expansion leaves the state vector unchanged while the bond grows; ahead of
    every single-site update (dmrg.jl:128-134) it lets DMRG from a D = 2 start reach the
    exact-diagonalisation energy."""
    L_ = 8
    H = M.finite_mpo_hamiltonian(L_, 2, M.heisenberg_terms(L_))
    psi = P.finite_mps_from_tensors(P.random_initial_tensors(L_, 2, 2, 6))
    assert psi.center == 0
    ac = psi.AC(0)
    Q, R = P.qr_pos(ac.reshape(-1, ac.shape[2], order="F"))
    psi.AL[0], psi.C[1], psi.center = Q.reshape(ac.shape, order="F"), R, 1
    v0 = _mps_vector(psi)
    D0 = psi.AR[2].shape[0]
    P.optimal_expand(1, True, psi, H, P.FiniteEnvironments(psi, H), P.OptimalExpand(3))
    assert psi.center == 2 and psi.AR[2].shape[0] > D0
    v1 = _mps_vector(psi)
    assert np.linalg.norm(v1 / np.linalg.norm(v1) - v0 / np.linalg.norm(v0)) < 1e-12
    L_ = 10
    H = M.finite_mpo_hamiltonian(L_, 2, M.heisenberg_terms(L_))
    e_ed = M.ed_ground_energy(L_, 2, M.heisenberg_terms(L_))[0]
    psi0 = P.finite_mps_from_tensors(P.random_initial_tensors(L_, 2, 2, 5))
    alg = P.DMRG(tol=1e-10, maxiter=12, alg_expand=P.OptimalExpand(4))
    _, _, eps, hist = P.find_groundstate_dmrg(psi0, H, alg)
    assert eps <= 1e-10
    assert abs(hist[-1][1] - e_ed) < 1e-10


@pytest.mark.parametrize("ov", [0, 2])
def test_oracle_sketched_expand_preserves_the_state_and_reaches_ed(ov):
    """SketchedExpand (changebonds/sketchedexpand.jl:75-162): the sketched directions are
    appended with zero weight (state unchanged, bond grown by `add`, orthonormal new rows
    orthogonal to the old ones), both directions; ahead of every single-site update it lets
    DMRG from a D = 2 start reach exact diagonalisation."""
    L_ = 8
    H = M.finite_mpo_hamiltonian(L_, 2, M.heisenberg_terms(L_))
    for right in (True, False):
        psi = P.finite_mps_from_tensors(P.random_initial_tensors(L_, 2, 2, 6))
        pos = 3
        # centre bond at pos (AC[pos] = C[pos] AR[pos]) with AL left of it
        psi_l = P.finite_mps_from_tensors(P.random_initial_tensors(L_, 2, 2, 6))
        for i in range(pos):
            A = np.einsum("ab,bsc->asc", psi_l.C[i], psi_l.AR[i])
            Q, R = P.qr_pos(A.reshape(-1, A.shape[2], order="F"))
            psi_l.AL[i] = Q.reshape(A.shape[0], 2, Q.shape[1], order="F")
            psi_l.C[i + 1] = R
            psi_l.center = i + 1
        psi = psi_l
        v0 = _mps_vector(psi)
        D0 = psi.C[pos].shape[0] if not right else psi.AR[pos + 1].shape[0]
        alg = P.SketchedExpand(2, oversampling=ov, seed=11)
        P.sketched_expand(pos, right, psi, H, P.FiniteEnvironments(psi, H), alg)
        v1 = _mps_vector(psi)
        assert np.linalg.norm(v1 / np.linalg.norm(v1) - v0 / np.linalg.norm(v0)) < 1e-12
        if right:
            D1 = psi.AR[pos + 1].shape[0]
            assert psi.center == pos + 1 and D1 == D0 + 2
            R_ = psi.AR[pos + 1].reshape(D1, -1, order="F")
            assert np.abs(R_ @ R_.conj().T - np.eye(D1)).max() < 1e-12
        else:
            D1 = psi.AL[pos - 1].shape[2]
            assert psi.center == pos and D1 == D0 + 2
            A_ = psi.AL[pos - 1].reshape(-1, D1, order="F")
            assert np.abs(A_.conj().T @ A_ - np.eye(D1)).max() < 1e-12
    L_ = 10
    H = M.finite_mpo_hamiltonian(L_, 2, M.heisenberg_terms(L_))
    e_ed = M.ed_ground_energy(L_, 2, M.heisenberg_terms(L_))[0]
    psi0 = P.finite_mps_from_tensors(P.random_initial_tensors(L_, 2, 2, 5))
    alg = P.DMRG(tol=1e-10, maxiter=12, alg_expand=P.SketchedExpand(4, oversampling=ov, seed=3))
    _, _, eps, hist = P.find_groundstate_dmrg(psi0, H, alg)
    assert abs(hist[-1][1] - e_ed) < 1e-9, (hist[-1][1], e_ed)


@pytest.mark.parametrize("right", [True, False])
def test_oracle_sketched_expand_with_a_full_sketch_is_optimal_expand(right):
    """A sketch spanning the whole complement (oversampling up to its dimension) makes the
    randomized selection of sketchedexpand.jl the exact one of optimalexpand.jl: the same
    enlarged bond space."""
    L_, pos = 8, 3
    H = M.finite_mpo_hamiltonian(L_, 2, M.heisenberg_terms(L_))
    As = P.random_initial_tensors(L_, 2, 3, 6)

    def centre():
        psi = P.finite_mps_from_tensors(As)
        for i in range(pos):
            A = np.einsum("ab,bsc->asc", psi.C[i], psi.AR[i])
            Q, R = P.qr_pos(A.reshape(-1, A.shape[2], order="F"))
            psi.AL[i], psi.C[i + 1] = Q.reshape(A.shape[0], 2, Q.shape[1], order="F"), R
            psi.center = i + 1
        return psi

    a, b = centre(), centre()
    P.sketched_expand(pos, right, a, H, P.FiniteEnvironments(a, H),
                      P.SketchedExpand(2, oversampling=8, seed=23))
    P.optimal_expand(pos, right, b, H, P.FiniteEnvironments(b, H), P.OptimalExpand(2))
    if right:
        x, y = (t.AR[pos + 1] for t in (a, b))
        x, y = (m.reshape(m.shape[0], -1, order="F") for m in (x, y))
    else:
        x, y = (t.AL[pos - 1] for t in (a, b))
        x, y = (m.reshape(-1, m.shape[2], order="F").T for m in (x, y))
    assert x.shape == y.shape
    assert np.abs(x.conj().T @ x - y.conj().T @ y).max() < 1e-10


def _state_vector(psi):
    """The state of an oracle FiniteMPS with its centre bond at psi.center."""
    T = np.ones((1, 1))
    for i in range(psi.center):
        T = np.tensordot(T, psi.AL[i], axes=([-1], [0]))
    T = np.tensordot(T, psi.C[psi.center], axes=([-1], [0]))
    for i in range(psi.center, len(psi)):
        T = np.tensordot(T, psi.AR[i], axes=([-1], [0]))
    return T.reshape(-1)


@pytest.mark.parametrize("kind", ["optimal", "sketched"])
def test_changebonds_grows_every_bond_and_keeps_the_state(kind):
    """changebonds!(psi, H, ::OptimalExpand / ::SketchedExpand) (optimalexpand.jl:191-199,
    sketchedexpand.jl:165-173): every bond with a nonempty complement grows by at most
    `add`, the state is unchanged and the left-canonical tensors stay isometric."""
    L_ = 8
    H = M.finite_mpo_hamiltonian(L_, 2, M.heisenberg_terms(L_))
    psi = P.finite_mps_from_tensors(P.random_initial_tensors(L_, 2, 3, 9))
    dims0 = [psi.C[b].shape[0] for b in range(1, L_)]
    v0 = _state_vector(psi)
    alg = P.OptimalExpand(2) if kind == "optimal" else P.SketchedExpand(2, seed=1)
    psi, _ = P.changebonds(psi, H, alg)
    assert psi.center == L_ - 1
    dims1 = [psi.AL[b].shape[2] for b in range(L_ - 1)]
    full = [min(2 ** (b + 1), 2 ** (L_ - b - 1)) for b in range(L_ - 1)]
    for a, b, f in zip(dims0, dims1, full):
        assert a <= b <= min(a + 2, f)
    assert sum(dims1) > sum(dims0)
    v1 = _state_vector(psi)
    assert abs(abs(np.vdot(v0, v1)) / (np.linalg.norm(v0) * np.linalg.norm(v1)) - 1) < 1e-12
    for b in range(L_ - 1):
        m = psi.AL[b].reshape(-1, psi.AL[b].shape[2], order="F")
        assert np.abs(m.conj().T @ m - np.eye(m.shape[1])).max() < 1e-12
