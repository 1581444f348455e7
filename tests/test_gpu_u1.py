"""U(1) symmetry on the device: block-wise gauge factorisations against the oracle, the
tile-skipping GEMM schedule against the dense one on block-sparse operators, and U(1) DMRG2
against the oracle."""
import numpy as np
import pytest

import mpsgb
from mpsgb import _lib as L
from mpsgb import u1 as HU
from mpsgb.operators import SPIN_HALF_CHARGES as QP
from oracle import mps as P
from oracle import u1 as U

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = mpsgb.context(0)
    yield c
    c.set_gemm_schedule("grouped", 0)
    c.set_svd_method("gesvd")


def _sym(rng, ql, qs, qr, dtype):
    a = rng.standard_normal((len(ql), len(qs), len(qr)))
    if np.dtype(dtype).kind == "c":
        a = a + 1j * rng.standard_normal(a.shape)
    return (a * HU.block_mask(ql, qs, qr)).astype(dtype)


def _charges(rng, n, lo=-3, hi=3):
    return np.sort(rng.integers(lo, hi + 1, size=n)).astype(np.int32)


@pytest.mark.parametrize("dt", [np.float64, np.complex128])
def test_u1_left_right_orth_match_oracle(ctx, dt):
    rng = np.random.default_rng(1)
    ql, qr = _charges(rng, 30), _charges(rng, 41)
    A = _sym(rng, ql, QP, qr, dt)
    t = mpsgb.DeviceTensor.from_numpy(ctx, "mps", A)
    t.charges = (ql, QP, qr)
    al, c = mpsgb.left_orth(t)
    Q, R, qk = U.left_orth_u1(A.reshape(-1, A.shape[2], order="F"), U.fuse(ql, QP), qr)
    assert np.array_equal(al.charges[2], qk)
    assert np.abs(al.numpy().reshape(Q.shape, order="F") - Q).max() < 1e-12
    assert np.abs(c.numpy() - R).max() < 1e-12
    # exact zeros outside the blocks
    assert np.all(al.numpy()[~HU.block_mask(ql, QP, qk)] == 0)
    cc, ar = mpsgb.right_orth(t)
    qcol = (qr[None, :] - QP[:, None]).reshape(-1, order="F")
    Lm, Q2, qk2 = U.right_orth_u1(A.reshape(A.shape[0], -1, order="F"), ql, qcol)
    assert np.array_equal(ar.charges[0], qk2)
    assert np.abs(ar.numpy().reshape(Q2.shape, order="F") - Q2).max() < 1e-12
    assert np.abs(cc.numpy() - Lm).max() < 1e-12
    assert np.all(ar.numpy()[~HU.block_mask(qk2, QP, qr)] == 0)


@pytest.mark.parametrize("method", ["gesvd", "gram"])
@pytest.mark.parametrize("dt", [np.float64, np.complex128])
def test_u1_svd_trunc_matches_oracle(ctx, method, dt):
    rng = np.random.default_rng(2)
    ql, qr = _charges(rng, 24, -2, 2), _charges(rng, 28, -2, 2)
    # AC2[l s1; r s2] with q_l + q_s1 + q_s2 = q_r
    a = rng.standard_normal((len(ql), 2, len(qr), 2))
    if np.dtype(dt).kind == "c":
        a = a + 1j * rng.standard_normal(a.shape)
    mask = HU.block_mask(ql, QP, qr, QP, signs=[1, 1, -1, 1])
    AC2 = (a * mask).astype(dt)
    ctx.set_svd_method(method)
    t = mpsgb.DeviceTensor.from_numpy(ctx, "ac2", AC2)
    t.charges = (ql, QP, qr, QP)
    for maxdim in (None, 17):
        al, S, ar, eps = mpsgb.svd_trunc(t, maxdim, 0.0, normalize=False)
        M_ = AC2.reshape(len(ql) * 2, -1, order="F")
        qcol = (qr[:, None] - QP[None, :]).reshape(-1, order="F")
        Uu, Sv, Vh, qk, oeps = U.svd_trunc_u1(M_, U.fuse(ql, QP), qcol, maxdim)
        assert np.array_equal(al.charges[2], qk)
        assert abs(eps - oeps) < 1e-10 * max(1.0, oeps)
        # same truncated matrix: AL C AR == U S Vh
        k = qk.size
        dev = np.einsum("lsk,km,mtr->lsrt", al.numpy(), S.numpy(), ar.numpy())
        ref = ((Uu * Sv) @ Vh).reshape(AC2.shape, order="F")
        assert np.abs(dev - ref).max() < 1e-10 * np.abs(ref).max()
        assert np.allclose(np.einsum("lsk,lsm->km", al.numpy().conj(), al.numpy()), np.eye(k),
                           atol=1e-11)
        assert np.all(al.numpy()[~HU.block_mask(ql, QP, qk)] == 0)
        assert np.all(ar.numpy()[~HU.block_mask(qk, QP, qr)] == 0)
    ctx.set_svd_method("gesvd")


def _u1_operator(ctx, L_=10, D=48, pos=4, seed=9, dtype=np.float64):
    H = mpsgb.heisenberg_XXX(L_, dtype=dtype, u1=True)
    As, qb = HU.random_u1_tensors(L_, D, seed, 0, dtype)
    psi = mpsgb.FiniteMPS.from_tensors(As, ctx, center=pos + 1, charges=(qb, QP))
    envs = mpsgb.FiniteEnvironments(psi, H)
    return psi, H, envs


@pytest.mark.parametrize("prec,tol", [("bf16x3", 1e-4), ("tf32x3", 4e-6)])
def test_tile_skipping_equals_dense_schedule_on_u1_operator(ctx, prec, tol):
    """Skipping k-blocks whose packed A and B tiles are zero changes nothing: the skipped
    products are exact zeros."""
    psi, H, envs = _u1_operator(ctx, L_=12, D=160, pos=5)
    be = mpsgb.GB300Backend(prec)
    ac2 = mpsgb.ac2_from(psi.AL[5], psi.ac(6))
    outs = {}
    for sched, bn in (("persistent", 0), ("persistent_dense", 0), ("persistent", 128),
                      ("tile", 0), ("grouped", 0)):
        ctx.set_gemm_schedule(sched, bn)
        Heff = mpsgb.AC2_hamiltonian(5, psi, H, envs, be)
        outs[(sched, bn)] = Heff(ac2).numpy()
    ctx.set_gemm_schedule("grouped", 0)
    ref = mpsgb.AC2_hamiltonian(5, psi, H, envs, mpsgb.GB300Backend("fp64"))(ac2).numpy()
    assert np.array_equal(outs[("persistent", 0)], outs[("persistent_dense", 0)])
    for v in outs.values():
        assert np.linalg.norm(v - ref) < tol * np.linalg.norm(ref)
    # H_eff preserves the block structure
    mask = HU.block_mask(psi.AL[5].charges[0], QP, psi.AR[6].charges[2], QP,
                         signs=[1, 1, -1, 1])
    assert np.all(ref[~mask] == 0)


def test_u1_dmrg2_matches_oracle(ctx):
    L_, D = 12, 32
    H = mpsgb.heisenberg_XXX(L_, dtype=np.float64, u1=True)
    As, qb = HU.random_u1_tensors(L_, D, 21, 0, np.float64)
    opsi = P.finite_mps_from_tensors(As, charges=(qb, QP))
    _, _, _, ohist = P.find_groundstate_dmrg2(opsi, H, P.DMRG2(maxdim=D, cutoff=1e-10),
                                              maxsweeps=5)
    psi = mpsgb.FiniteMPS.from_tensors(As, ctx, charges=(qb, QP))
    psi, envs, eps, hist = mpsgb.find_groundstate(psi, H, mpsgb.DMRG2(maxdim=D, cutoff=1e-10),
                                                  maxsweeps=5)
    for a, b in zip(hist, ohist):
        assert abs(a["energy"] - b[1]) < 1e-10 * abs(b[1]), (a, b)


@pytest.mark.parametrize("prec,bar", [("tf32x3", 1e-9), ("bf16x3", 2e-9)])
def test_u1_dmrg2_split_precision_gram(ctx, prec, bar):
    """Split-precision contractions + Gram factorisation per block reach the FP64 oracle
    energy of the same U(1) run.  tf32x3 (22 significant bits per operand pair) lands within
    ~1e-12; bf16x3 (16 bits) carries an energy error of ~1e-9 on this 16-site chain (measured
    3e-10 to 1.3e-9 over GEMM schedules, factorisations and sweep counts): the error of the
    variational energy is quadratic in the operator's, ~(2^-16)^2 against (2^-22)^2."""
    L_, D = 16, 48
    H = mpsgb.heisenberg_XXX(L_, dtype=np.float64, u1=True)
    As, qb = HU.random_u1_tensors(L_, D, 23, 0, np.float64)
    opsi = P.finite_mps_from_tensors(As, charges=(qb, QP))
    _, _, _, ohist = P.find_groundstate_dmrg2(opsi, H, P.DMRG2(maxdim=D, cutoff=1e-12),
                                              maxsweeps=8)
    ctx.set_svd_method("gram")
    ctx.set_precision(prec)
    try:
        psi = mpsgb.FiniteMPS.from_tensors(As, ctx, charges=(qb, QP))
        alg = mpsgb.DMRG2(maxdim=D, cutoff=1e-12, backend=mpsgb.GB300Backend(prec))
        psi, envs, eps, hist = mpsgb.find_groundstate(psi, H, alg, maxsweeps=8)
        # the FP64 refinement step: energy from FP64 environments of the converged state
        e = mpsgb.expectation_value(psi, H, mpsgb.FiniteEnvironments(psi, H), 0)
    finally:
        ctx.set_svd_method("gesvd")
        ctx.set_precision("fp64")
    e_ref = ohist[-1][1]
    assert abs(e - e_ref) < bar * abs(e_ref), (e, e_ref)


@pytest.mark.parametrize("prec", ["bf16x3", "tf32x3"])
def test_sector_restricted_chain_is_exact(ctx, prec):
    """gb_heff_set_sectors: the fused AA chain of a U(1) J1-J2 operator computes only the
    charge-allowed entries of its intermediate; the result is bit-for-bit the one of the
    same operator without sectors (AC2 and one-site AC, two applications each)."""
    L_, pos = 12, 5
    H = mpsgb.j1j2_cylinder(4, 3, u1=True)
    As, qb = HU.random_u1_tensors(L_, 96, 13, 0, np.float64)
    psi = mpsgb.FiniteMPS.from_tensors(As, ctx, center=pos + 1, charges=(qb, QP))
    envs = mpsgb.FiniteEnvironments(psi, H)
    be = mpsgb.GB300Backend(prec)
    ctx.set_gemm_schedule("persistent", 0)  # the restricted chain of the dense-embedding path
    try:
        _restricted_chain_checks(ctx, psi, H, envs, be, pos)
    finally:
        ctx.set_gemm_schedule("grouped", 0)


def _restricted_chain_checks(ctx, psi, H, envs, be, pos):
    ac2 = mpsgb.ac2_from(psi.AL[pos], psi.ac(pos + 1))
    plain = ac2.copy()
    plain.charges = None  # the same vector without its leg charges: no sectors
    Hs = mpsgb.AC2_hamiltonian(pos, psi, H, envs, be)
    assert "AA" in Hs.terms
    ys = [Hs(ac2).numpy() for _ in range(2)]
    assert Hs._sectors is not None
    yd = mpsgb.AC2_hamiltonian(pos, psi, H, envs, be)(plain).numpy()
    assert np.array_equal(ys[0], yd) and np.array_equal(ys[1], yd)
    ac = psi.ac(pos + 1)
    Hs1 = mpsgb.AC_hamiltonian(pos + 1, psi, H, envs, be)
    y1 = Hs1(ac).numpy()
    assert Hs1._sectors is not None
    ac_plain = ac.copy()
    ac_plain.charges = None
    y1d = mpsgb.AC_hamiltonian(pos + 1, psi, H, envs, be)(ac_plain).numpy()
    assert np.array_equal(y1, y1d)
    # unsorted left charges are refused
    bad = mpsgb.AC2_hamiltonian(pos, psi, H, envs, be)
    q = [np.ascontiguousarray(c, dtype=np.int32) for c in ac2.charges]
    q0 = q[0][::-1].copy()
    if np.any(np.diff(q0) < 0):
        p = lambda a: a.ctypes.data_as(L.PI32)
        with pytest.raises(RuntimeError):
            L.check(L.lib().gb_heff_set_sectors(bad.handle, p(q0), p(q[1]), p(q[3]), p(q[2])))


def test_compact_krylov_matches_dense_solves(ctx):
    """With the sectors known, eigsolve and exponentiate keep only the charge-allowed entries
    of their vectors; eigenvalue, eigenvector and exp(-i dt H) x agree with the solves on the
    full charge-sorted embedding (FP64; only the summation order differs)."""
    L_, pos = 10, 4
    H = mpsgb.heisenberg_XXX(L_, dtype=np.complex128, u1=True)
    As, qb = HU.random_u1_tensors(L_, 40, 17, 0, np.complex128)
    psi = mpsgb.FiniteMPS.from_tensors(As, ctx, center=pos + 1, charges=(qb, QP))
    envs = mpsgb.FiniteEnvironments(psi, H)
    be = mpsgb.GB300Backend("fp64")
    ac2 = mpsgb.ac2_from(psi.AL[pos], psi.ac(pos + 1))
    plain = ac2.copy()
    plain.charges = None
    alg = mpsgb.Lanczos(krylovdim=30, maxiter=100, tol=1e-12, eager=True)
    Hs = mpsgb.AC2_hamiltonian(pos, psi, H, envs, be)
    Hd = mpsgb.AC2_hamiltonian(pos, psi, H, envs, be)
    ls, xs, infs = mpsgb.fixedpoint(Hs, ac2, "SR", alg)
    ld, xd, infd = mpsgb.fixedpoint(Hd, plain, "SR", alg)
    assert Hs._sectors is not None and Hd._sectors is None
    assert abs(ls - ld) < 1e-12 * abs(ld)
    a, b = xs.numpy(), xd.numpy()
    assert abs(abs(np.vdot(a, b)) - 1.0) < 1e-10
    mask = HU.block_mask(psi.AL[pos].charges[0], QP, psi.AR[pos + 1].charges[2], QP,
                         signs=[1, 1, -1, 1])
    assert np.all(a[~mask] == 0)
    ys = mpsgb.integrate(Hs, ac2, 0.0, 0.1, mpsgb.Lanczos(tol=1e-12)).numpy()
    yd = mpsgb.integrate(Hd, plain, 0.0, 0.1, mpsgb.Lanczos(tol=1e-12)).numpy()
    assert np.linalg.norm(ys - yd) < 1e-10 * np.linalg.norm(yd)


def _grouped_vs_fp64(ctx, psi, H, envs, pos, prec, tol, two_site=True):
    """One operator on the grouped schedule (default) and on the dense-embedding schedule,
    against the FP64 operator: two applications each."""
    be = mpsgb.GB300Backend(prec)
    if two_site:
        x = mpsgb.ac2_from(psi.AL[pos], psi.ac(pos + 1))
        make = lambda b: mpsgb.AC2_hamiltonian(pos, psi, H, envs, b)
    else:
        x = psi.ac(pos)
        make = lambda b: mpsgb.AC_hamiltonian(pos, psi, H, envs, b)
    ref = make(mpsgb.GB300Backend("fp64"))(x).numpy()
    ctx.set_gemm_schedule("grouped", 0)
    Hg = make(be)
    yg = [Hg(x).numpy() for _ in range(2)]
    ctx.set_gemm_schedule("persistent", 0)
    try:
        yp = make(be)(x).numpy()
    finally:
        ctx.set_gemm_schedule("grouped", 0)
    nref = np.linalg.norm(ref)
    for y in yg + [yp]:
        assert np.linalg.norm(y - ref) < tol * nref, (prec, np.linalg.norm(y - ref) / nref)
    # the same result on every call (operands repacked, the mix output reused)
    assert np.array_equal(yg[0], yg[1])
    # exact zeros outside the charge blocks
    assert np.all(yg[0][ref == 0] == 0)
    return Hg


@pytest.mark.parametrize("prec,tol", [("bf16x3", 1e-4), ("tf32x3", 4e-6)])
@pytest.mark.parametrize("model", ["j1j2", "heisenberg"])
def test_grouped_sector_gemm_matches_fp64(ctx, prec, tol, model):
    """The grouped sector-block GEMMs (one launch per contraction over its charge blocks,
    block-stacked operands, per-block tile widths): two-site and one-site operators of a
    long-range (AA, CA, AB terms) and a nearest-neighbour (IC, BE terms) U(1) model agree
    with the FP64 operator within the split-precision tolerance."""
    L_, pos = 12, 5
    if model == "j1j2":
        H = mpsgb.j1j2_cylinder(4, 3, u1=True)
        D = 96
    else:
        H = mpsgb.heisenberg_XXX(L_, dtype=np.float64, u1=True)
        D = 160
    As, qb = HU.random_u1_tensors(L_, D, 31, 0, np.float64)
    psi = mpsgb.FiniteMPS.from_tensors(As, ctx, center=pos + 1, charges=(qb, QP))
    envs = mpsgb.FiniteEnvironments(psi, H)
    Hg = _grouped_vs_fp64(ctx, psi, H, envs, pos, prec, tol, two_site=True)
    if model == "j1j2":
        assert "AA" in Hg.terms
    else:
        assert "IC" in Hg.terms and "BE" in Hg.terms
    _grouped_vs_fp64(ctx, psi, H, envs, pos + 1, prec, tol, two_site=False)


def test_grouped_counts_the_same_nonzero_products(ctx):
    """Counting mode: the grouped GEMMs report the same block-sparse product count as the
    dense-embedding GEMMs, and execute far fewer tile products."""
    L_, pos = 12, 5
    H = mpsgb.j1j2_cylinder(4, 3, u1=True)
    As, qb = HU.random_u1_tensors(L_, 128, 37, 0, np.float64)
    psi = mpsgb.FiniteMPS.from_tensors(As, ctx, center=pos + 1, charges=(qb, QP))
    envs = mpsgb.FiniteEnvironments(psi, H)
    x = mpsgb.ac2_from(psi.AL[pos], psi.ac(pos + 1))
    be = mpsgb.GB300Backend("bf16x3")
    work = {}
    try:
        for sched in ("grouped", "persistent"):
            ctx.set_gemm_schedule(sched, 0)
            # counting on before the build: the dense-embedding path counts its constant
            # operands when it packs them
            ctx.set_counting(True)
            Heff = mpsgb.AC2_hamiltonian(pos, psi, H, envs, be)
            Heff.set_sectors(x)
            ctx.synchronize()
            ctx.read_work(reset=True)
            Heff(x)
            ctx.synchronize()
            ctx.set_counting(False)
            work[sched] = ctx.read_work(reset=True)
    finally:
        ctx.set_counting(False)
        ctx.set_gemm_schedule("grouped", 0)
    g, p = work["grouped"], work["persistent"]
    assert g["nonzero_flops"] > 0
    assert abs(g["nonzero_flops"] - p["nonzero_flops"]) <= 1e-9 * p["nonzero_flops"]
    assert g["tile_flops"] < p["tile_flops"]


@pytest.mark.parametrize("prec", ["bf16x3", "tf32x3"])
def test_staged_chain_mix_is_bitwise_the_plain_mix(ctx, prec):
    """The grouped schedule's chain mix staged through shared memory (per column and charge
    of the rows, GB_OPT_STAGED_MIX) sums in the same order as the plain per-row form: the
    operator's output is bit-for-bit the same, AC2 and one-site AC."""
    L_, pos = 12, 5
    H = mpsgb.j1j2_cylinder(4, 3, u1=True)
    As, qb = HU.random_u1_tensors(L_, 96, 13, 0, np.float64)
    psi = mpsgb.FiniteMPS.from_tensors(As, ctx, center=pos + 1, charges=(qb, QP))
    envs = mpsgb.FiniteEnvironments(psi, H)
    be = mpsgb.GB300Backend(prec)
    ac2 = mpsgb.ac2_from(psi.AL[pos], psi.ac(pos + 1))
    ac = psi.ac(pos + 1)
    out = {}
    for staged in (2, 0):
        ctx.set_option("staged_mix", staged)
        try:
            H2 = mpsgb.AC2_hamiltonian(pos, psi, H, envs, be)
            H1 = mpsgb.AC_hamiltonian(pos + 1, psi, H, envs, be)
            out[staged] = (H2(ac2).numpy(), H1(ac).numpy())
        finally:
            ctx.set_option("staged_mix", 1)
    assert "AA" in H2.terms
    assert np.array_equal(out[2][0], out[0][0]) and np.array_equal(out[2][1], out[0][1])


def test_grouped_split_k_is_deterministic_and_accurate(ctx):
    """Long-K sector blocks run as split-K units whose FP32 partial sums the last unit adds
    in unit order: repeated applications are bit-for-bit identical, and the result agrees
    with the FP64 operator to the split-precision tolerance."""
    L_, pos = 24, 11
    H = mpsgb.j1j2_cylinder(6, 4, u1=True)
    As, qb = HU.random_u1_tensors(L_, 512, 43, 0, np.float64)
    psi = mpsgb.FiniteMPS.from_tensors(As, ctx, center=pos + 1, charges=(qb, QP))
    envs = mpsgb.FiniteEnvironments(psi, H)
    x = mpsgb.ac2_from(psi.AL[pos], psi.ac(pos + 1))
    op = mpsgb.AC2_hamiltonian(pos, psi, H, envs, mpsgb.GB300Backend("bf16x3"))
    ys = [op(x).numpy() for _ in range(3)]
    desc = op.describe()
    assert any("split_tiles=" in l and "split_tiles=0" not in l for l in desc.splitlines()), desc
    assert np.array_equal(ys[0], ys[1]) and np.array_equal(ys[0], ys[2])
    ref = mpsgb.AC2_hamiltonian(pos, psi, H, envs, mpsgb.GB300Backend("fp64"))(x).numpy()
    assert np.linalg.norm(ys[0] - ref) < 1e-4 * np.linalg.norm(ref)


def test_packed_environments_are_exact_and_small(ctx):
    """gb_tensor_pack keeps only the nonzero 64 x 64 tiles of a U(1) environment's dense
    embedding and gb_packed_unpack restores it bit for bit; FiniteEnvironments(packed=True)
    serves the same environments as the dense cache."""
    L_, pos = 24, 11
    H = mpsgb.heisenberg_XXX(L_, dtype=np.float64, u1=True)
    As, qb = HU.random_u1_tensors(L_, 1024, 47, 0, np.float64)
    psi = mpsgb.FiniteMPS.from_tensors(As, ctx, center=pos + 1, charges=(qb, QP))
    dense = mpsgb.FiniteEnvironments(psi, H)
    packed = mpsgb.FiniteEnvironments(psi, H, packed=True)
    for i in range(pos - 2, pos + 1):
        a = dense.leftenv(i, psi).numpy()
        b = packed.leftenv(i, psi).numpy()
        assert np.array_equal(a, b)
    GL = dense.leftenv(pos, psi)
    p = mpsgb.core.PackedTensor(GL)
    kept, total, nbytes = p.info()
    assert kept < total and nbytes < 0.5 * GL.numpy().nbytes
    assert np.array_equal(p.unpack().numpy(), GL.numpy())
    # every environment but the requested one is held packed
    assert sum(isinstance(g, mpsgb.core.PackedTensor) for g in packed.GL) >= pos - 1
    for i in (pos + 3, pos + 2, pos + 1):
        assert np.array_equal(dense.rightenv(i, psi).numpy(), packed.rightenv(i, psi).numpy())
    # an environment asked for again comes back from its packed copy
    assert np.array_equal(dense.leftenv(pos - 1, psi).numpy(), packed.leftenv(pos - 1, psi).numpy())
