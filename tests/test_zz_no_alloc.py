"""The allocation-free bond-operator entry point (gb_c_apply_noalloc).

Callers that cannot allocate device memory -- an external Krylov solver whose arrays all
come from its own pool, or launches recorded into a CUDA graph -- pass their own device
buffers; the library's only intermediate lives in a fixed 64 MiB device array.  This test
calls it through the C ABI on torch-owned buffers and checks it against the regular
operator entry point (gb_heff_build(GB_HEFF_C) + gb_heff_apply) on two calls in a row.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12  # relative, same FP64 arithmetic on both paths


def _envs():
    from oracle import models as M
    from oracle import mps as P
    L_ = 10
    H = M.finite_mpo_hamiltonian(L_, 2, M.xxz_terms(L_, 1.0, 0.7, 0.2))
    psi = P.finite_mps_from_tensors(P.random_initial_tensors(L_, 2, 24, 55))
    envs = P.FiniteEnvironments(psi, H)
    pos = 4
    return envs.leftenv(pos + 1, psi), envs.rightenv(pos, psi)


def test_c_apply_noalloc_matches_operator_entry_point():
    torch = pytest.importorskip("torch")
    import mpsgb
    from mpsgb import _lib as L

    ctx = mpsgb.context(0)
    GL, GR = _envs()                       # reference leg order: GL[a, w, a'], GR[b', w, b]
    Dl, w, Dr = GL.shape[0], GL.shape[1], GR.shape[0]
    op = mpsgb.DerivativeOperator(ctx, L.GB_HEFF_C, mpsgb.DeviceTensor.from_numpy(ctx, "gl", GL),
                                  None, None, mpsgb.DeviceTensor.from_numpy(ctx, "gr", GR),
                                  mpsgb.GB300Backend("fp64"))
    dev = torch.device("cuda", 0)
    # caller-owned buffers in the device layouts: GL (a, a', w), GR (b', w, b), x (l, r),
    # all column-major, i.e. C-order arrays with the axes reversed
    tGL = torch.from_numpy(np.ascontiguousarray(GL.transpose(1, 2, 0))).to(dev)
    tGR = torch.from_numpy(np.ascontiguousarray(GR.transpose(2, 1, 0))).to(dev)
    rng = np.random.default_rng(3)
    for call in range(2):
        x = rng.standard_normal((Dl, Dr)) + 1j * rng.standard_normal((Dl, Dr))
        tx = torch.from_numpy(np.ascontiguousarray(x.T)).to(dev)
        ty = torch.empty((Dr, Dl), dtype=torch.complex128, device=dev)
        stream = torch.cuda.current_stream(dev).cuda_stream
        rc = L.lib().gb_c_apply_noalloc(ctypes.c_void_p(tGL.data_ptr()),
                                        ctypes.c_void_p(tGR.data_ptr()),
                                        ctypes.c_void_p(tx.data_ptr()),
                                        ctypes.c_void_p(ty.data_ptr()), Dl, Dr, w, L.GB_C128,
                                        ctypes.c_void_p(stream))
        assert rc == L.GB_OK, L.lib().gb_last_error()
        torch.cuda.synchronize(dev)
        y_new = ty.cpu().numpy().T
        y_ref = op(mpsgb.DeviceTensor.from_numpy(ctx, "bond", x)).numpy()
        err = np.linalg.norm(y_new - y_ref) / np.linalg.norm(y_ref)
        assert err < FP64_TOL, (call, err)


def test_c_apply_noalloc_rejects_oversize_problems():
    """Sizes beyond the static scratch are refused on the host before any launch."""
    from mpsgb import _lib as L
    dummy = ctypes.c_void_p(16)  # never dereferenced: the size check comes first
    rc = L.lib().gb_c_apply_noalloc(dummy, dummy, dummy, dummy, 4096, 4096, 64, L.GB_F64, None)
    assert rc == L.GB_ERR_ARG
    assert b"static scratch" in L.lib().gb_last_error()
