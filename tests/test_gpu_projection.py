"""Projections between different bra and ket states (C/AC/AC2_projection with below != above,
src/algorithms/derivatives/derivatives.jl:194-216, through the generic MPO operators of
mpo_derivatives.jl:37-66) against the oracle: rectangular environments, and environments
built between two different states by the device transfers."""
import numpy as np
import pytest

import mpsgb
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
def test_rectangular_projections_match_the_oracle(ctx, dt):
    rng = np.random.default_rng(51)
    Dlb, Dlk, Drk, Drb, d, wl, wm, wr = 14, 10, 12, 9, 2, 4, 5, 3
    GL = _rand(rng, (Dlb, wl, Dlk), dt)
    GR = _rand(rng, (Drk, wr, Drb), dt)
    W1 = _rand(rng, (wl, d, d, wm), dt)
    W2 = _rand(rng, (wm, d, d, wr), dt)
    W = _rand(rng, (wl, d, d, wr), dt)
    dGL = mpsgb.DeviceTensor.from_numpy(ctx, "gl", GL)
    dGR = mpsgb.DeviceTensor.from_numpy(ctx, "gr", GR)
    # C (the environments share their channel count)
    GRc = _rand(rng, (Drk, wl, Drb), dt)
    xc = _rand(rng, (Dlk, Drk), dt)
    y = mpsgb.mpo_projection(dGL, mpsgb.DeviceTensor.from_numpy(ctx, "gr", GRc),
                             mpsgb.DeviceTensor.from_numpy(ctx, "bond", xc)).numpy()
    assert y.shape == (Dlb, Drb) and _rel(y, dv.mpo_c_apply(GL, GRc, xc)) < 1e-13
    # AC
    x1 = _rand(rng, (Dlk, d, Drk), dt)
    y = mpsgb.mpo_projection(dGL, dGR, mpsgb.DeviceTensor.from_numpy(ctx, "mps", x1), W).numpy()
    assert y.shape == (Dlb, d, Drb) and _rel(y, dv.mpo_ac_apply(GL, W, GR, x1)) < 1e-13
    # AC2
    x2 = _rand(rng, (Dlk, d, Drk, d), dt)
    y = mpsgb.mpo_projection(dGL, dGR, mpsgb.DeviceTensor.from_numpy(ctx, "ac2", x2), W1,
                             W2).numpy()
    assert y.shape == (Dlb, d, Drb, d)
    assert _rel(y, dv.mpo_ac2_apply(GL, W1, W2, GR, x2)) < 1e-13


def test_projection_between_two_states(ctx):
    """AC2_projection(site, below, H, above): environments from the transfers with the bra
    the state `below` and the ket `above` (gb_env_transfer_left/right with A != Abar)."""
    L_, pos, dt = 8, 3, np.complex128
    H = M.finite_mpo_hamiltonian(L_, 2, M.heisenberg_terms(L_))
    below = P.finite_mps_from_tensors(P.random_initial_tensors(L_, 2, 6, 61))
    above = P.finite_mps_from_tensors(P.random_initial_tensors(L_, 2, 5, 62))
    # oracle environments of <below| H |above> in right-canonical tensors
    GL = np.ones((1, 1, 1), dtype=dt)
    for j in range(pos):
        GL = dv.transfer_left(GL, H[j], above.AR[j], below.AR[j])
    GR = np.ones((1, 1, 1), dtype=dt)
    for j in range(L_ - 1, pos + 1, -1):
        GR = dv.transfer_right(GR, H[j], above.AR[j], below.AR[j])
    x = np.einsum("asm,mtb->asbt", above.AR[pos], above.AR[pos + 1])
    ref = dv.mpo_ac2_apply(GL, H[pos], H[pos + 1], GR, x)
    # the same on the device, through the public transfers with bra != ket
    T = lambda kind, a: mpsgb.DeviceTensor.from_numpy(ctx, kind, a)
    g = T("gl", np.ones((1, 1, 1), dtype=dt))
    for j in range(pos):
        g = mpsgb.transfer_left(g, H[j], T("mps", above.AR[j]), T("mps", below.AR[j]))
    r = T("gr", np.ones((1, 1, 1), dtype=dt))
    for j in range(L_ - 1, pos + 1, -1):
        r = mpsgb.transfer_right(r, H[j], T("mps", above.AR[j]), T("mps", below.AR[j]))
    assert np.abs(g.numpy() - GL).max() < 1e-12 and np.abs(r.numpy() - GR).max() < 1e-12
    y = mpsgb.mpo_projection(g, r, T("ac2", x), H[pos], H[pos + 1]).numpy()
    assert y.shape == ref.shape and _rel(y, ref) < 1e-12
