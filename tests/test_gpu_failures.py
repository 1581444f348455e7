"""Failure paths of the device engine, made without any GPU fault.

* A bounded wait that runs out: every mbarrier wait of the tensor-core kernels is bounded
  (gb_ctx_set_wait_bound); with the bound at zero the first wait that is not already
  satisfied gives up, the kernel records GB_ERR_TIMEOUT, drains the copies and MMAs it has
  issued, frees its tensor memory and returns.  The host reads the status, restores the
  bound and the same context computes correctly again.
* Non-finite data: a NaN in the environment or in the start vector is caught by the FP64
  norms of the Lanczos solve (KrylovKit's residual check of
  src/algorithms/fixedpoint.jl:15-23) and reported as GB_ERR_NAN.
* Non-convergence is not an error: maxiter = 1 with an unreachable tolerance returns the
  best Ritz pair with info.converged = 0 (KrylovKit ConvergenceInfo semantics, read by
  src/algorithms/groundstate/dmrg.jl:153)."""
import numpy as np
import pytest

import mpsgb
from mpsgb import _lib as L

pytestmark = pytest.mark.gpu


def _operator(ctx, prec, D=256, seed=3, poison=False):
    H = mpsgb.j1j2_cylinder(6, 3)
    pos = len(H) // 2 - 1
    W = H.device(ctx)
    rng = np.random.default_rng(seed)
    wl, wr = H.W[pos].shape[0], H.W[pos + 1].shape[3]
    GL = rng.standard_normal((D, wl, D))
    GR = rng.standard_normal((D, wr, D))
    if poison:
        GL[D // 3, 1, D // 2] = np.nan
    dGL = mpsgb.DeviceTensor.from_numpy(ctx, "gl", GL)
    dGR = mpsgb.DeviceTensor.from_numpy(ctx, "gr", GR)
    op = mpsgb.DerivativeOperator(ctx, L.GB_HEFF_AC2, dGL, W[pos], W[pos + 1], dGR,
                                  mpsgb.GB300Backend(prec))
    x = rng.standard_normal(op.xdims)
    return op, x, (dGL, dGR, W)


def test_wait_timeout_is_reported_and_the_context_recovers():
    ctx = mpsgb.Context(0)
    op, x, keep = _operator(ctx, "bf16x3")
    ref_op, _, keep2 = _operator(ctx, "fp64")
    xd = mpsgb.DeviceTensor.from_numpy(ctx, "ac2", x)
    ref = ref_op(xd).numpy()
    assert ctx.device_status() == 0
    ctx.set_wait_bound(0.0)
    try:
        op(xd)
        ctx.synchronize()
        status = ctx.device_status()
    finally:
        ctx.set_wait_bound(2.0)
    assert status == L.GB_ERR_TIMEOUT
    # the same context, the same operator: correct again, status clean
    y = op(xd).numpy()
    ctx.synchronize()
    assert ctx.device_status() == 0
    assert np.linalg.norm(y - ref) < 1e-4 * np.linalg.norm(ref)


def test_wait_timeout_in_the_grouped_kernel():
    """The same for the grouped sector-block GEMM (a U(1) operator with known sectors)."""
    from mpsgb import u1 as HU
    from mpsgb.operators import SPIN_HALF_CHARGES as QP
    ctx = mpsgb.Context(0)
    L_, pos = 18, 8
    H = mpsgb.j1j2_cylinder(6, 3, u1=True)
    As, qb = HU.random_u1_tensors(L_, 256, 41, 0, np.float64)
    psi = mpsgb.FiniteMPS.from_tensors(As, ctx, center=pos + 1, charges=(qb, QP))
    envs = mpsgb.FiniteEnvironments(psi, H)
    x = mpsgb.ac2_from(psi.AL[pos], psi.ac(pos + 1))
    ref = mpsgb.AC2_hamiltonian(pos, psi, H, envs, mpsgb.GB300Backend("fp64"))(x).numpy()
    op = mpsgb.AC2_hamiltonian(pos, psi, H, envs, mpsgb.GB300Backend("bf16x3"))
    op.set_sectors(x)
    ctx.synchronize()
    assert ctx.device_status() == 0
    ctx.set_wait_bound(0.0)
    try:
        op(x)
        ctx.synchronize()
        status = ctx.device_status()
    finally:
        ctx.set_wait_bound(2.0)
    assert status == L.GB_ERR_TIMEOUT
    y = op(x).numpy()
    ctx.synchronize()
    assert ctx.device_status() == 0
    assert np.linalg.norm(y - ref) < 1e-4 * np.linalg.norm(ref)


def test_nan_in_environment_is_reported():
    ctx = mpsgb.context(0)
    op, x, keep = _operator(ctx, "fp64", D=48, poison=True)
    with pytest.raises(L.GBError) as e:
        mpsgb.fixedpoint(op, mpsgb.DeviceTensor.from_numpy(ctx, "ac2", x), "SR",
                         mpsgb.Lanczos(krylovdim=8, maxiter=2, tol=1e-10))
    assert e.value.code == L.GB_ERR_NAN


def test_nan_in_start_vector_is_reported():
    ctx = mpsgb.context(0)
    op, x, keep = _operator(ctx, "fp64", D=48)
    x.flat[7] = np.nan
    with pytest.raises(L.GBError) as e:
        mpsgb.fixedpoint(op, mpsgb.DeviceTensor.from_numpy(ctx, "ac2", x), "SR",
                         mpsgb.Lanczos(krylovdim=8, maxiter=2, tol=1e-10))
    assert e.value.code == L.GB_ERR_NAN


def test_forced_non_convergence_is_not_an_error():
    ctx = mpsgb.context(0)
    L_ = 10
    H = mpsgb.heisenberg_XXX(L_, dtype=np.float64)
    As = mpsgb.states.random_tensors(L_, 2, 16, seed=5, dtype=np.float64)
    psi = mpsgb.FiniteMPS.from_tensors(As, ctx, center=5)
    envs = mpsgb.FiniteEnvironments(psi, H)
    Heff = mpsgb.AC2_hamiltonian(4, psi, H, envs, mpsgb.GB300Backend("fp64"))
    x0 = mpsgb.ac2_from(psi.AL[4], psi.ac(5))
    val, vec, info = mpsgb.fixedpoint(Heff, x0, "SR",
                                      mpsgb.Lanczos(krylovdim=3, maxiter=1, tol=1e-14))
    assert info.converged == 0
    assert info.numops == 3 and info.normres > 1e-14
    assert np.isfinite(val)
    # the returned vector is the normalised best Ritz vector
    assert abs(vec.norm() - 1.0) < 1e-12
