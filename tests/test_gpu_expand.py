"""Bond expansion on the device against the oracle: the DMRG3S perturbation
(post_expand/dmrg3s.jl:133-192), concatenation along a bond, the two-sided complement
projection, OptimalExpand (changebonds/optimalexpand.jl:122-187), SketchedExpand
(changebonds/sketchedexpand.jl:75-162) and single-site DMRG with each expansion from a D = 2
start (the oracle reaches exact diagonalisation with both,
tests/test_oracle.py)."""
import numpy as np
import pytest

import mpsgb
from mpsgb import _lib as L
from oracle import derivatives as dv
from oracle import models as M
from oracle import mps as P

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    return mpsgb.context(0)


def _rand(rng, shape, dt):
    x = rng.standard_normal(shape)
    if np.dtype(dt).kind == "c":
        x = x + 1j * rng.standard_normal(shape)
    return x.astype(dt)


def _rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.mark.parametrize("dt", [np.float64, np.complex128])
def test_perturbation_matches_the_combiner_contraction(ctx, dt):
    rng = np.random.default_rng(41)
    Dl, Dr, d, wl, wr = 12, 10, 2, 5, 4
    GL = _rand(rng, (Dl + 3, wl, Dl), dt)    # bra bond Dl + 3, ket Dl
    GR = _rand(rng, (Dr, wr, Dr + 2), dt)
    W = _rand(rng, (wl, d, d, wr), dt)
    AC = _rand(rng, (Dl, d, Dr), dt)
    dac = mpsgb.DeviceTensor.from_numpy(ctx, "mps", AC)
    dW = mpsgb.DeviceTensor.from_numpy(ctx, "mpo", W)
    # side 0: combiner[r, w, (r w)] as a GR-like right environment (bond fastest)
    comb = np.zeros((Dr, wr, Dr * wr), dtype=dt)
    for w in range(wr):
        comb[np.arange(Dr), w, w * Dr + np.arange(Dr)] = 1
    ref = dv.mpo_ac_apply(GL, W, comb, AC)
    got = mpsgb.states.perturb(mpsgb.DeviceTensor.from_numpy(ctx, "gl", GL), dW, dac, 0).numpy()
    assert got.shape == ref.shape and _rel(got, ref) < 1e-13
    # side 1: combiner[(l w), w, l] as a GL-like left environment
    comb = np.zeros((Dl * wl, wl, Dl), dtype=dt)
    for w in range(wl):
        comb[w * Dl + np.arange(Dl), w, np.arange(Dl)] = 1
    ref = dv.mpo_ac_apply(comb, W, GR, AC)
    got = mpsgb.states.perturb(mpsgb.DeviceTensor.from_numpy(ctx, "gr", GR), dW, dac, 1).numpy()
    assert got.shape == ref.shape and _rel(got, ref) < 1e-13


def test_cat_reshape_and_right_complement(ctx):
    rng = np.random.default_rng(42)
    A = rng.standard_normal((6, 2, 5))
    B = rng.standard_normal((6, 2, 3))
    C = rng.standard_normal((4, 2, 5))
    dA = mpsgb.DeviceTensor.from_numpy(ctx, "mps", A)
    cat = mpsgb.states.mps_cat
    assert np.array_equal(cat(dA, mpsgb.DeviceTensor.from_numpy(ctx, "mps", B), 2).numpy(),
                          np.concatenate([A, B], axis=2))
    assert np.array_equal(cat(dA, mpsgb.DeviceTensor.from_numpy(ctx, "mps", C), 0).numpy(),
                          np.concatenate([A, C], axis=0))
    assert np.array_equal(cat(dA, None, 2, nb=4).numpy(),
                          np.concatenate([A, np.zeros((6, 2, 4))], axis=2))
    assert np.array_equal(cat(dA, None, 0, nb=3).numpy(),
                          np.concatenate([A, np.zeros((3, 2, 5))], axis=0))
    # an MPS tensor is the two-site tensor (Dl, d, Dr, 1) over the same storage
    t = dA.copy().reshape_(L.GB_KIND_AC2, (6, 2, 5, 1))
    assert np.array_equal(t.numpy()[..., 0], A)
    t = dA.copy().reshape_(L.GB_KIND_AC2, (6, 1, 5, 2))
    assert np.array_equal(t.numpy()[:, 0].transpose(0, 2, 1), A)
    # Y <- Y (1 - X' X) on the trailing (s2, r) legs of a two-site tensor
    Q, _ = np.linalg.qr(rng.standard_normal((2 * 7, 3)))
    X = Q.T.reshape(3, 2, 7, order="F")                       # orthonormal rows
    Y = rng.standard_normal((5, 2, 7, 2))                      # (l, s1, r, s2)
    Ym = Y.transpose(0, 1, 3, 2).reshape(10, 14, order="F")    # (l s1) x (s2 r)
    Xm = X.reshape(3, 14, order="F")
    ref = (Ym - (Ym @ Xm.T) @ Xm).reshape(5, 2, 2, 7, order="F").transpose(0, 1, 3, 2)
    dY = mpsgb.DeviceTensor.from_numpy(ctx, "ac2", Y)
    mpsgb.states.project_complement_right_(dY, mpsgb.DeviceTensor.from_numpy(ctx, "mps", X))
    assert np.abs(dY.numpy() - ref).max() < 1e-13


def _vector(ts):
    v = ts[0]
    for t in ts[1:]:
        v = np.tensordot(v, t, axes=([v.ndim - 1], [0]))
    return v.reshape(-1)


def test_optimal_expand_matches_the_oracle(ctx):
    L_ = 8
    H = M.finite_mpo_hamiltonian(L_, 2, M.heisenberg_terms(L_))
    As = P.random_initial_tensors(L_, 2, 2, 6)
    # oracle: centre bond moved to 1, then the expansion of bond (1, 2)
    opsi = P.finite_mps_from_tensors(As)
    ac = opsi.AC(0)
    Q, R = P.qr_pos(ac.reshape(-1, ac.shape[2], order="F"))
    opsi.AL[0], opsi.C[1], opsi.center = Q.reshape(ac.shape, order="F"), R, 1
    oenv = P.FiniteEnvironments(opsi, H)
    D0 = opsi.AR[2].shape[0]
    P.optimal_expand(1, True, opsi, H, oenv, P.OptimalExpand(3))
    # device: the same steps
    Hd = mpsgb.heisenberg_XXX(L_)
    psi = mpsgb.FiniteMPS.from_tensors(As, ctx)
    q, Rd = mpsgb.left_orth(psi.ac(0))
    psi.AL[0], psi.C[1], psi.center = q, Rd, 1
    v0 = _vector([psi.AL[0].numpy(), psi.ac(1).numpy()] + [psi.AR[i].numpy() for i in range(2, L_)])
    envs = mpsgb.FiniteEnvironments(psi, Hd)
    mpsgb.algorithms.optimal_expand(1, True, psi, Hd, envs, mpsgb.OptimalExpand(3))
    assert psi.center == 2
    assert psi.AR[2].dims == opsi.AR[2].shape and psi.AR[2].dims[0] > D0
    v1 = _vector([psi.AL[0].numpy(), psi.AL[1].numpy(), psi.ac(2).numpy()]
                 + [psi.AR[i].numpy() for i in range(3, L_)])
    assert np.linalg.norm(v1 / np.linalg.norm(v1) - v0 / np.linalg.norm(v0)) < 1e-12
    # the same added directions (rows of AR[2] beyond D0, up to a sign per row)
    new_d = psi.AR[2].numpy()[D0:].reshape(-1, 2 * opsi.AR[2].shape[2], order="F")
    new_o = opsi.AR[2][D0:].reshape(-1, 2 * opsi.AR[2].shape[2], order="F")
    assert np.abs(new_d @ new_d.conj().T - np.eye(new_d.shape[0])).max() < 1e-12
    assert np.abs(new_d.conj().T @ new_d - new_o.conj().T @ new_o).max() < 1e-10


@pytest.mark.parametrize("right", [True, False])
@pytest.mark.parametrize("ov", [0, 2])
def test_sketched_expand_matches_the_oracle(ctx, right, ov):
    """SketchedExpand (sketchedexpand.jl:75-162) with the same random sketch: the same bond
    growth and added directions, the state unchanged."""
    L_, pos = 8, 3
    As = P.random_initial_tensors(L_, 2, 3, 6)
    Hd = mpsgb.heisenberg_XXX(L_)
    psi = mpsgb.FiniteMPS.from_tensors(As, ctx, center=pos)
    # the oracle state in the device state's gauge, and the device MPO's channel basis
    n = lambda t: None if t is None else t.numpy()
    opsi = P.FiniteMPS([n(psi.AL[i]) if i < pos else None for i in range(L_)],
                       [n(psi.AR[i]) if i >= pos else None for i in range(L_)],
                       [n(psi.C[i]) if i == pos else None for i in range(L_ + 1)], pos)
    H = M.MPOHam([np.asarray(w, dtype=np.complex128) for w in Hd.W], Hd.chans)
    P.sketched_expand(pos, right, opsi, H, P.FiniteEnvironments(opsi, H),
                      P.SketchedExpand(2, oversampling=ov, seed=23))
    full = lambda ps: _vector([ps.AL[i].numpy() for i in range(ps.center)]
                              + [ps.ac(ps.center).numpy()]
                              + [ps.AR[i].numpy() for i in range(ps.center + 1, L_)])
    v0 = full(psi)
    envs = mpsgb.FiniteEnvironments(psi, Hd)
    mpsgb.algorithms.sketched_expand(pos, right, psi, Hd, envs,
                                     mpsgb.SketchedExpand(2, oversampling=ov, seed=23))
    assert psi.center == opsi.center
    v1 = full(psi)
    assert np.linalg.norm(v1 / np.linalg.norm(v1) - v0 / np.linalg.norm(v0)) < 1e-12
    if right:
        a, b = psi.AR[pos + 1].numpy(), opsi.AR[pos + 1]
        a, b = (x.reshape(x.shape[0], -1, order="F") for x in (a, b))
    else:
        a, b = psi.AL[pos - 1].numpy(), opsi.AL[pos - 1]
        a, b = (x.reshape(-1, x.shape[2], order="F").T for x in (a, b))
    assert a.shape == b.shape
    if ov == 0:
        assert np.abs(a - b).max() < 1e-10          # QR / LQ: the same rows
    else:
        assert np.abs(a.conj().T @ a - b.conj().T @ b).max() < 1e-10   # SVD: the same span


@pytest.mark.parametrize("kind", ["optimal_expand", "dmrg3s", "sketched_expand"])
def test_single_site_dmrg_with_expansion_reaches_ed(ctx, kind):
    L_ = 10
    terms = M.heisenberg_terms(L_)
    oH = M.finite_mpo_hamiltonian(L_, 2, terms)
    e_ed = M.ed_ground_energy(L_, 2, terms)[0]
    As = P.random_initial_tensors(L_, 2, 2, 5)
    if kind == "optimal_expand":
        oalg = P.DMRG(tol=1e-10, maxiter=12, alg_expand=P.OptimalExpand(4))
        alg = mpsgb.DMRG(tol=1e-10, maxiter=12, alg_expand=mpsgb.OptimalExpand(4))
        bar = 1e-10
    elif kind == "sketched_expand":
        oalg = P.DMRG(tol=1e-10, maxiter=12, alg_expand=P.SketchedExpand(4, seed=3))
        alg = mpsgb.DMRG(tol=1e-10, maxiter=12, alg_expand=mpsgb.SketchedExpand(4, seed=3))
        bar = 1e-9
    else:
        oalg = P.DMRG(tol=1e-10, maxiter=12, alg_gauge=P.DMRG3S(0.1, 0.8, 16, 1e-12))
        alg = mpsgb.DMRG(tol=1e-10, maxiter=12, alg_gauge=mpsgb.DMRG3S(0.1, 0.8, 16, 1e-12))
        bar = 1e-7
    _, _, _, ohist = P.find_groundstate_dmrg(P.finite_mps_from_tensors(As), oH, oalg)
    psi = mpsgb.FiniteMPS.from_tensors(As, ctx)
    psi, envs, eps, hist = mpsgb.find_groundstate(psi, mpsgb.heisenberg_XXX(L_), alg)
    assert len(hist) == len(ohist)
    for a, b in zip(hist, ohist):
        assert abs(a["energy"] - b[1]) <= 1e-8 * abs(b[1]), (a, b)
    assert -1e-12 * abs(e_ed) <= hist[-1]["energy"] - e_ed < bar


@pytest.mark.parametrize("right", [True, False])
def test_u1_optimal_expand_keeps_the_state_and_sorted_bond(ctx, right):
    """OptimalExpand on a U(1) state: the SVD of the projected two-site update runs per charge
    block and the enlarged bond is re-sorted by charge (gb_mps_permute); the state vector is
    unchanged, the bond grows, its charges stay sorted and the new tensors are isometries."""
    from mpsgb import u1 as HU
    from mpsgb.operators import SPIN_HALF_CHARGES as QP
    L_, pos = 8, 3
    H = mpsgb.heisenberg_XXX(L_, dtype=np.float64, u1=True)
    As, qb = HU.random_u1_tensors(L_, 2, 31, 0, np.float64)
    psi = mpsgb.FiniteMPS.from_tensors(As, ctx, center=pos, charges=(qb, QP))
    full = lambda ps: _vector([ps.AL[i].numpy() for i in range(ps.center)]
                              + [ps.ac(ps.center).numpy()]
                              + [ps.AR[i].numpy() for i in range(ps.center + 1, L_)])
    v0 = full(psi)
    D0 = psi.C[pos].dims[0]
    mpsgb.algorithms.optimal_expand(pos, right, psi, H, mpsgb.FiniteEnvironments(psi, H),
                                    mpsgb.OptimalExpand(3))
    v1 = full(psi)
    assert np.linalg.norm(v1 / np.linalg.norm(v1) - v0 / np.linalg.norm(v0)) < 1e-12
    if right:
        A = psi.AR[pos + 1]
        q = A.charges[0]
        m = A.numpy().reshape(A.dims[0], -1, order="F")
        assert np.abs(m @ m.T - np.eye(A.dims[0])).max() < 1e-12
        assert psi.center == pos + 1 and A.dims[0] > 2
        assert np.array_equal(psi.AL[pos].charges[2], q)
    else:
        A = psi.AL[pos - 1]
        q = A.charges[2]
        m = A.numpy().reshape(-1, A.dims[2], order="F")
        assert np.abs(m.T @ m - np.eye(A.dims[2])).max() < 1e-12
        assert psi.center == pos and A.dims[2] > D0
        assert np.array_equal(psi.AR[pos].charges[0], q)
    assert np.all(np.diff(q) >= 0)
    # every entry outside the charge blocks is exactly zero
    ql, qs, qr = A.charges
    mask = HU.block_mask(ql, qs, qr)
    assert np.all(A.numpy()[~mask] == 0)


def test_u1_single_site_dmrg_with_optimal_expand_reaches_ed(ctx):
    from mpsgb import u1 as HU
    from mpsgb.operators import SPIN_HALF_CHARGES as QP
    L_ = 10
    terms = M.heisenberg_terms(L_)
    e_ed = M.ed_ground_energy(L_, 2, terms)[0]
    As, qb = HU.random_u1_tensors(L_, 2, 5, 0, np.float64)
    psi = mpsgb.FiniteMPS.from_tensors(As, ctx, charges=(qb, QP))
    alg = mpsgb.DMRG(tol=1e-10, maxiter=12, alg_expand=mpsgb.OptimalExpand(4))
    psi, envs, eps, hist = mpsgb.find_groundstate(psi, mpsgb.heisenberg_XXX(L_, dtype=np.float64,
                                                                            u1=True), alg)
    assert -1e-12 * abs(e_ed) <= hist[-1]["energy"] - e_ed < 1e-9 * abs(e_ed), (hist[-1], e_ed)


def _u1_blocks_ok(psi):
    """Every stored site tensor of a U(1) state is exactly zero outside its charge blocks and
    its bonds are sorted by charge."""
    from mpsgb import u1 as HU
    for i in range(len(psi.AL)):
        A = psi.AL[i] if i < psi.center else psi.AR[i]
        ql, qs, qr = A.charges
        assert np.all(np.diff(ql) >= 0) and np.all(np.diff(qr) >= 0)
        assert np.all(A.numpy()[~HU.block_mask(ql, qs, qr)] == 0), i


@pytest.mark.parametrize("kind", ["dmrg3s", "sketched_expand", "sketched_oversampled"])
def test_u1_single_site_dmrg_with_expansion_matches_the_oracle(ctx, kind):
    """U(1) DMRG3S (the perturbation's fused leg labelled by q_bond + q_channel) and U(1)
    SketchedExpand (per-sector sketch) from a D = 2 start: the sweep energies follow the
    oracle's, the state reaches exact diagonalisation and stays block sparse."""
    from mpsgb import u1 as HU
    from mpsgb.operators import SPIN_HALF_CHARGES as QP
    L_ = 10
    e_ed = M.ed_ground_energy(L_, 2, M.heisenberg_terms(L_, dtype=np.float64))[0]
    As, qb = HU.random_u1_tensors(L_, 2, 5, 0, np.float64)
    H = mpsgb.heisenberg_XXX(L_, dtype=np.float64, u1=True)
    if kind == "dmrg3s":
        oalg = P.DMRG(tol=1e-10, maxiter=12, alg_gauge=P.DMRG3S(0.1, 0.8, 16, 1e-12))
        alg = mpsgb.DMRG(tol=1e-10, maxiter=12, alg_gauge=mpsgb.DMRG3S(0.1, 0.8, 16, 1e-12))
        bar = 1e-7
    else:
        ov = 2 if kind == "sketched_oversampled" else 0
        oalg = P.DMRG(tol=1e-10, maxiter=12, alg_expand=P.SketchedExpand(4, ov, seed=3))
        alg = mpsgb.DMRG(tol=1e-10, maxiter=12, alg_expand=mpsgb.SketchedExpand(4, ov, seed=3))
        bar = 1e-9
    _, _, _, ohist = P.find_groundstate_dmrg(P.finite_mps_from_tensors(As, charges=(qb, QP)),
                                             H, oalg)
    psi = mpsgb.FiniteMPS.from_tensors(As, ctx, charges=(qb, QP))
    psi, envs, eps, hist = mpsgb.find_groundstate(psi, H, alg)
    assert len(hist) == len(ohist)
    for a, b in zip(hist, ohist):
        assert abs(a["energy"] - b[1]) <= 1e-8 * abs(b[1]), (a, b)
    assert -1e-12 * abs(e_ed) <= hist[-1]["energy"] - e_ed < bar * abs(e_ed)
    _u1_blocks_ok(psi)


@pytest.mark.parametrize("kind", ["optimal", "sketched"])
def test_changebonds_matches_the_oracle(ctx, kind):
    """changebonds!(psi, H, ::OptimalExpand / ::SketchedExpand) (optimalexpand.jl:191-199,
    sketchedexpand.jl:165-173) over a whole chain: the same enlarged bonds as the oracle and
    the same (unchanged) state."""
    L_ = 8
    As = P.random_initial_tensors(L_, 2, 3, 9)
    oH = M.finite_mpo_hamiltonian(L_, 2, M.heisenberg_terms(L_))
    oalg = P.OptimalExpand(2) if kind == "optimal" else P.SketchedExpand(2, seed=1)
    alg = mpsgb.OptimalExpand(2) if kind == "optimal" else mpsgb.SketchedExpand(2, seed=1)
    opsi, _ = P.changebonds(P.finite_mps_from_tensors(As), oH, oalg)
    psi, _ = mpsgb.changebonds(mpsgb.FiniteMPS.from_tensors(As, ctx), mpsgb.heisenberg_XXX(L_),
                               alg)
    assert psi.center == L_ - 1
    assert [psi.AL[b].dims[2] for b in range(L_ - 1)] == \
        [opsi.AL[b].shape[2] for b in range(L_ - 1)]
    v = _vector([psi.AL[b].numpy() for b in range(L_ - 1)] + [psi.ac(L_ - 1).numpy()])
    ov = _vector([opsi.AL[b] for b in range(L_ - 1)] + [opsi.ac(L_ - 1)])
    assert abs(abs(np.vdot(v, ov)) / (np.linalg.norm(v) * np.linalg.norm(ov)) - 1) < 1e-10
