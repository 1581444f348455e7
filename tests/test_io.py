"""The interchange archives (mpsgb.io): an MPO round-trips exactly on the host; a state and
its environments round-trip through the device bit for bit and resume a DMRG2 run that
reaches the energy of the uninterrupted one."""
import numpy as np
import pytest

import mpsgb
from mpsgb import io as IO
from mpsgb import u1 as HU
from mpsgb.operators import SPIN_HALF_CHARGES as QP


@pytest.mark.parametrize("build", ["heis_u1", "j1j2", "tfim_inf"])
def test_mpo_round_trip(tmp_path, build):
    H = {"heis_u1": lambda: mpsgb.heisenberg_XXX(8, dtype=np.float64, u1=True),
         "j1j2": lambda: mpsgb.j1j2_cylinder(4, 3),
         "tfim_inf": lambda: mpsgb.transverse_field_ising(1, g=0.7, infinite=True)}[build]()
    path = str(tmp_path / "h.npz")
    IO.save_mpo(path, H)
    G = IO.load_mpo(path)
    assert G.finite == H.finite and len(G) == len(H)
    for a, b in zip(G.W, H.W):
        assert a.dtype == b.dtype and np.array_equal(a, b)
    assert (G.chans is None) == (H.chans is None)
    if H.chans is not None:
        for a, b in zip(G.chans, H.chans):
            assert np.array_equal(np.asarray(a), np.asarray(b))


def test_mpo_archive_is_checked(tmp_path):
    path = str(tmp_path / "bad.npz")
    np.savez(path, kind=np.array("mpo"), finite=np.array(True), nsites=np.array(2),
             W0=np.zeros((1, 2, 2, 3)), W1=np.zeros((4, 2, 2, 1)))
    with pytest.raises(ValueError):
        IO.load_mpo(path)
    np.savez(path, kind=np.array("finite_mps"), nsites=np.array(1))
    with pytest.raises(ValueError):
        IO.load_mpo(path)


@pytest.mark.gpu
def test_state_and_environments_resume_a_sweep(tmp_path):
    ctx = mpsgb.context(0)
    L_, D = 12, 32
    H = mpsgb.heisenberg_XXX(L_, dtype=np.float64, u1=True)
    As, qb = HU.random_u1_tensors(L_, D, 29, 0, np.float64)
    alg = mpsgb.DMRG2(maxdim=D, cutoff=1e-12)
    # uninterrupted: 3 sweeps
    psi = mpsgb.FiniteMPS.from_tensors(As, ctx, charges=(qb, QP))
    _, _, _, h3 = mpsgb.find_groundstate(psi, H, alg, maxsweeps=3)
    # 1 sweep, archive state and environments, reload, 2 more sweeps
    psi = mpsgb.FiniteMPS.from_tensors(As, ctx, charges=(qb, QP))
    psi, envs, _, h1 = mpsgb.find_groundstate(psi, H, alg, maxsweeps=1)
    IO.save_state(str(tmp_path / "s.npz"), psi)
    IO.save_environments(str(tmp_path / "e.npz"), envs)
    p2 = IO.load_state(str(tmp_path / "s.npz"), ctx)
    assert p2.center == psi.center
    for i in range(L_):
        a = psi.AL[i] if i < psi.center else psi.AR[i]
        b = p2.AL[i] if i < p2.center else p2.AR[i]
        assert np.array_equal(a.numpy(), b.numpy())
        assert all(np.array_equal(x, y) for x, y in zip(a.charges, b.charges))
    e2 = IO.load_environments(str(tmp_path / "e.npz"), p2, H, ctx)
    _, _, _, hr = mpsgb.find_groundstate(p2, H, alg, envs=e2, maxsweeps=2)
    # the first sweep is the same computation; the resumed run restarts the adaptive
    # Krylov budgets (find_groundstate! keeps no error history), so later sweeps agree to
    # convergence rather than bitwise
    assert h1[0]["energy"] == h3[0]["energy"]
    assert len(hr) >= 1
    assert abs(hr[-1]["energy"] - h3[-1]["energy"]) <= 1e-8 * abs(h3[-1]["energy"])
