"""GPU parity of the derivative operators (through the C ABI) against the oracle."""
import os

import numpy as np
import pytest

import mpsgb
from mpsgb import _lib as L
from oracle import derivatives as dv
from oracle import models as M
from oracle import mps as P

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
FP64_TOL = 1e-12      # relative, plain FP64 path
SPLIT_TOL = 1e-4      # relative, bf16x3 split path (hi/lo BF16 operands, FP32 accumulate)
TF32_TOL = 4e-6       # relative, tf32x3 split path (hi/lo TF32 operands, FP32 accumulate)


@pytest.fixture(scope="module")
def ctx():
    return mpsgb.context(0)


def _envs(L_, terms, dt, D, seed):
    H = M.finite_mpo_hamiltonian(L_, 2, terms, dtype=dt)
    psi = P.finite_mps_from_tensors(P.random_initial_tensors(L_, 2, D, seed, dt))
    return H, psi, P.FiniteEnvironments(psi, H)


def _rand(rng, shape, dt):
    x = rng.standard_normal(shape)
    if np.dtype(dt).kind == "c":
        x = x + 1j * rng.standard_normal(shape)
    return x.astype(dt)


def _rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def dev_op(ctx, kind, GL, W1, W2, GR, prec="fp64"):
    dt = GL.dtype
    g = mpsgb.DeviceTensor.from_numpy(ctx, "gl", GL)
    r = mpsgb.DeviceTensor.from_numpy(ctx, "gr", GR)
    w1 = mpsgb.DeviceTensor.from_numpy(ctx, "mpo", W1) if W1 is not None else None
    w2 = mpsgb.DeviceTensor.from_numpy(ctx, "mpo", W2) if W2 is not None else None
    return mpsgb.DerivativeOperator(ctx, kind, g, w1, w2, r, mpsgb.GB300Backend(prec))


@pytest.mark.parametrize("name", ["ac2_heisenberg_c128", "ac2_tfim_edge_f64", "ac2_j1j2_f64"])
def test_ac2_golden_fixtures(ctx, name):
    f = np.load(os.path.join(HERE, "golden", f"{name}.npz"))
    op = dev_op(ctx, L.GB_HEFF_AC2, f["GL"], f["W1"], f["W2"], f["GR"])
    assert ",".join(op.terms) == str(f["terms"])
    y = op(mpsgb.DeviceTensor.from_numpy(ctx, "ac2", f["x"])).numpy()
    assert _rel(y, f["y"]) < FP64_TOL


MODELS = {
    "heis_c": lambda: (10, M.heisenberg_terms(10), np.complex128),
    "heis_r": lambda: (10, M.heisenberg_terms(10, dtype=np.float64), np.float64),
    "tfim_r": lambda: (9, M.tfim_terms(9, g=0.9, dtype=np.float64), np.float64),
    "xxz_field_c": lambda: (9, M.xxz_terms(9, 1.0, 1.5, 0.25), np.complex128),
    "j1j2_r": lambda: (12, M.j1j2_cylinder_terms(4, 3), np.float64),
}


@pytest.mark.parametrize("model", sorted(MODELS))
def test_ac2_every_bond(ctx, model):
    L_, terms, dt = MODELS[model]()
    H, psi, envs = _envs(L_, terms, dt, 12, 21)
    rng = np.random.default_rng(5)
    for pos in range(L_ - 1):
        GL, GR = envs.leftenv(pos, psi), envs.rightenv(pos + 1, psi)
        op = dev_op(ctx, L.GB_HEFF_AC2, GL, H[pos], H[pos + 1], GR)
        ref_op = dv.JordanAC2(GL, H[pos], H[pos + 1], GR)
        assert op.terms == ref_op.terms(), (pos, op.terms, ref_op.terms())
        x = _rand(rng, (GL.shape[0], 2, GR.shape[0], 2), dt)
        y = op(mpsgb.DeviceTensor.from_numpy(ctx, "ac2", x)).numpy()
        assert _rel(y, ref_op(x)) < FP64_TOL, (model, pos)


@pytest.mark.parametrize("model", sorted(MODELS))
def test_ac_every_site(ctx, model):
    L_, terms, dt = MODELS[model]()
    H, psi, envs = _envs(L_, terms, dt, 12, 22)
    rng = np.random.default_rng(6)
    for pos in range(L_):
        GL, GR = envs.leftenv(pos, psi), envs.rightenv(pos, psi)
        op = dev_op(ctx, L.GB_HEFF_AC, GL, H[pos], None, GR)
        ref_op = dv.JordanAC(GL, H[pos], GR)
        x = _rand(rng, (GL.shape[0], 2, GR.shape[0]), dt)
        y = op(mpsgb.DeviceTensor.from_numpy(ctx, "mps", x)).numpy()
        assert _rel(y, ref_op(x)) < FP64_TOL, (model, pos)


@pytest.mark.parametrize("model", ["heis_c", "j1j2_r"])
def test_c_every_bond(ctx, model):
    L_, terms, dt = MODELS[model]()
    H, psi, envs = _envs(L_, terms, dt, 12, 23)
    rng = np.random.default_rng(7)
    for pos in range(L_ - 1):
        GL, GR = envs.leftenv(pos + 1, psi), envs.rightenv(pos, psi)
        op = dev_op(ctx, L.GB_HEFF_C, GL, None, None, GR)
        x = _rand(rng, (GL.shape[0], GR.shape[0]), dt)
        y = op(mpsgb.DeviceTensor.from_numpy(ctx, "bond", x)).numpy()
        assert _rel(y, dv.mpo_c_apply(GL, GR, x)) < FP64_TOL


@pytest.mark.parametrize("model", ["heis_c", "heis_r", "j1j2_r"])
def test_split_precision_apply(ctx, model):
    L_, terms, dt = MODELS[model]()
    H, psi, envs = _envs(L_, terms, dt, 32, 24)
    rng = np.random.default_rng(8)
    pos = L_ // 2 - 1
    GL, GR = envs.leftenv(pos, psi), envs.rightenv(pos + 1, psi)
    op = dev_op(ctx, L.GB_HEFF_AC2, GL, H[pos], H[pos + 1], GR, "bf16x3")
    x = _rand(rng, (GL.shape[0], 2, GR.shape[0], 2), dt)
    y = op(mpsgb.DeviceTensor.from_numpy(ctx, "ac2", x)).numpy()
    err = _rel(y, dv.JordanAC2(GL, H[pos], H[pos + 1], GR)(x))
    assert err < SPLIT_TOL, err
    assert ctx.device_status() == 0


@pytest.mark.parametrize("model", ["heis_c", "j1j2_r"])
def test_tf32_split_precision_apply(ctx, model):
    """hi/lo TF32 operands: products exact in FP32, so the error left is the FP32
    accumulation of the tensor pipe (~1e-6 here) -- below the BF16 split error, which adds
    a 2^-16 representation error per operand."""
    L_, terms, dt = MODELS[model]()
    H, psi, envs = _envs(L_, terms, dt, 32, 24)
    rng = np.random.default_rng(9)
    pos = L_ // 2 - 1
    GL, GR = envs.leftenv(pos, psi), envs.rightenv(pos + 1, psi)
    x = _rand(rng, (GL.shape[0], 2, GR.shape[0], 2), dt)
    ref = dv.JordanAC2(GL, H[pos], H[pos + 1], GR)(x)
    errs = {}
    for prec in ("bf16x3", "tf32x3"):
        op = dev_op(ctx, L.GB_HEFF_AC2, GL, H[pos], H[pos + 1], GR, prec)
        errs[prec] = _rel(op(mpsgb.DeviceTensor.from_numpy(ctx, "ac2", x)).numpy(), ref)
    assert errs["tf32x3"] < TF32_TOL, errs
    assert errs["tf32x3"] < errs["bf16x3"], errs
    # switching an existing operator's precision repacks its constant operands
    op.set_precision("bf16x3")
    e = _rel(op(mpsgb.DeviceTensor.from_numpy(ctx, "ac2", x)).numpy(), ref)
    assert abs(e - errs["bf16x3"]) < 1e-3 * errs["bf16x3"] + 1e-15
    assert ctx.device_status() == 0


def test_linearity_of_apply(ctx):
    """H(a x + b z) = a H(x) + b H(z) on the device (size-independent property)."""
    L_, terms, dt = MODELS["xxz_field_c"]()
    H, psi, envs = _envs(L_, terms, dt, 16, 25)
    pos = 3
    GL, GR = envs.leftenv(pos, psi), envs.rightenv(pos + 1, psi)
    op = dev_op(ctx, L.GB_HEFF_AC2, GL, H[pos], H[pos + 1], GR)
    rng = np.random.default_rng(9)
    shape = (GL.shape[0], 2, GR.shape[0], 2)
    x, z = _rand(rng, shape, dt), _rand(rng, shape, dt)
    a, b = 0.3 - 1.2j, 2.1 + 0.4j
    dx = mpsgb.DeviceTensor.from_numpy(ctx, "ac2", x)
    dz = mpsgb.DeviceTensor.from_numpy(ctx, "ac2", z)
    lhs = op(mpsgb.DeviceTensor.from_numpy(ctx, "ac2", a * x + b * z)).numpy()
    rhs = a * op(dx).numpy() + b * op(dz).numpy()
    assert _rel(lhs, rhs) < 1e-13


def test_hermiticity(ctx):
    L_, terms, dt = MODELS["heis_c"]()
    H, psi, envs = _envs(L_, terms, dt, 8, 26)
    pos = 4
    GL, GR = envs.leftenv(pos, psi), envs.rightenv(pos + 1, psi)
    op = dev_op(ctx, L.GB_HEFF_AC2, GL, H[pos], H[pos + 1], GR)
    rng = np.random.default_rng(10)
    shape = (GL.shape[0], 2, GR.shape[0], 2)
    x, z = _rand(rng, shape, dt), _rand(rng, shape, dt)
    hx = op(mpsgb.DeviceTensor.from_numpy(ctx, "ac2", x)).numpy()
    hz = op(mpsgb.DeviceTensor.from_numpy(ctx, "ac2", z)).numpy()
    assert abs(np.vdot(z, hx) - np.conj(np.vdot(x, hz))) < 1e-11 * np.linalg.norm(hx)


def test_errors_are_reported_not_crashing(ctx):
    f = np.load(os.path.join(HERE, "golden", "ac2_heisenberg_c128.npz"))
    op = dev_op(ctx, L.GB_HEFF_AC2, f["GL"], f["W1"], f["W2"], f["GR"])
    wrong = mpsgb.DeviceTensor(ctx, "ac2", np.complex128, (3, 2, 3, 2))
    with pytest.raises(L.GBError) as e:
        op(wrong)
    assert e.value.code == L.GB_ERR_ARG


def test_launch_trace_accounts_every_launch(ctx):
    """gb_ctx_trace_begin/end: one event per launch site visit (a site may issue two
    kernels), charged to named source sites; the per-site times add up to the span."""
    L_, terms, dt = MODELS["heis_c"]()
    H, psi, envs = _envs(L_, terms, dt, 16, 26)
    pos = 3
    GL, GR = envs.leftenv(pos, psi), envs.rightenv(pos + 1, psi)
    op = dev_op(ctx, L.GB_HEFF_AC2, GL, H[pos], H[pos + 1], GR, "bf16x3")
    x = mpsgb.DeviceTensor.from_numpy(ctx, "ac2", _rand(np.random.default_rng(3),
                                                        (GL.shape[0], 2, GR.shape[0], 2), dt))
    op(x)
    ctx.synchronize()
    n0 = ctx.kernel_launches()
    ctx.trace_begin()
    op(x)
    span, sites = ctx.trace_end()
    launches = ctx.kernel_launches() - n0
    assert launches > 0 and sites
    assert 0 < sum(ev for _, _, ev in sites) <= launches
    assert all(":" in nm and nm.split(":")[0].endswith(".cu") for nm, _, _ in sites)
    assert abs(sum(ms for _, ms, _ in sites) - span) <= 1e-3 * max(span, 1.0) + 1e-3


# ------------------------------------------------------------------ generic MPO operators
# MPO_AC_Hamiltonian / MPO_AC2_Hamiltonian of an arbitrary MPO (mpo_derivatives.jl:46-66,
# 100-107, 144-153): dense W with no Jordan structure, every channel pair contracted.

def _generic_case(rng, dt, D=24, wl=3, wm=4, wr=3, d=2):
    GL = _rand(rng, (D, wl, D), dt)
    GR = _rand(rng, (D + 4, wr, D + 4), dt)
    W1 = _rand(rng, (wl, d, d, wm), dt)
    W2 = _rand(rng, (wm, d, d, wr), dt)
    return GL, W1, W2, GR


@pytest.mark.parametrize("dt", [np.float64, np.complex128])
@pytest.mark.parametrize("prec,tol", [("fp64", FP64_TOL), ("bf16x3", SPLIT_TOL)])
def test_generic_mpo_ac2(ctx, dt, prec, tol):
    if prec != "fp64" and dt == np.complex128:
        pytest.skip("split precision contracts real data")
    rng = np.random.default_rng(31)
    GL, W1, W2, GR = _generic_case(rng, dt)
    op = dev_op(ctx, L.GB_HEFF_AC2_MPO, GL, W1, W2, GR, prec)
    assert op.terms == ("AA",)
    x = _rand(rng, (GL.shape[0], 2, GR.shape[0], 2), dt)
    y = op(mpsgb.DeviceTensor.from_numpy(ctx, "ac2", x)).numpy()
    assert _rel(y, dv.mpo_ac2_apply(GL, W1, W2, GR, x)) < tol


@pytest.mark.parametrize("dt", [np.float64, np.complex128])
@pytest.mark.parametrize("prec,tol", [("fp64", FP64_TOL), ("bf16x3", SPLIT_TOL)])
def test_generic_mpo_ac(ctx, dt, prec, tol):
    if prec != "fp64" and dt == np.complex128:
        pytest.skip("split precision contracts real data")
    rng = np.random.default_rng(32)
    GL, W1, _, GR = _generic_case(rng, dt, wr=4)
    op = dev_op(ctx, L.GB_HEFF_AC_MPO, GL, W1, None, GR, prec)
    assert op.terms == ("A",)
    x = _rand(rng, (GL.shape[0], 2, GR.shape[0]), dt)
    y = op(mpsgb.DeviceTensor.from_numpy(ctx, "mps", x)).numpy()
    assert _rel(y, dv.mpo_ac_apply(GL, W1, GR, x)) < tol


def test_generic_form_of_a_hamiltonian_equals_the_jordan_form(ctx):
    """On a Jordan-form Hamiltonian MPO the generic operator (all channel pairs) and the
    prepared Jordan operator are the same linear map."""
    L_, terms, dt = MODELS["j1j2_r"]()
    H, psi, envs = _envs(L_, terms, dt, 12, 23)
    rng = np.random.default_rng(7)
    pos = 5
    GL, GR = envs.leftenv(pos, psi), envs.rightenv(pos + 1, psi)
    x = _rand(rng, (GL.shape[0], 2, GR.shape[0], 2), dt)
    xd = mpsgb.DeviceTensor.from_numpy(ctx, "ac2", x)
    yj = dev_op(ctx, L.GB_HEFF_AC2, GL, H[pos], H[pos + 1], GR)(xd).numpy()
    yg = dev_op(ctx, L.GB_HEFF_AC2_MPO, GL, H[pos], H[pos + 1], GR)(xd).numpy()
    assert _rel(yg, yj) < FP64_TOL
    GR1 = envs.rightenv(pos, psi)
    x1 = _rand(rng, (GL.shape[0], 2, GR1.shape[0]), dt)
    x1d = mpsgb.DeviceTensor.from_numpy(ctx, "mps", x1)
    yj = dev_op(ctx, L.GB_HEFF_AC, GL, H[pos], None, GR1)(x1d).numpy()
    yg = dev_op(ctx, L.GB_HEFF_AC_MPO, GL, H[pos], None, GR1)(x1d).numpy()
    assert _rel(yg, yj) < FP64_TOL
