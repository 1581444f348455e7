"""Generate the oracle fixtures in tests/golden (run from the repository root):

    python tests/golden/make_golden.py

Each fixture holds a seeded MPO site pair, environments, an input vector and the
oracle's output of the Jordan-form derivative operator (hamiltonian_derivatives.jl),
plus an exact-diagonalisation energy.  The oracle itself is pinned by the reference's
known answers in known_answers.json (see tests/test_oracle.py).
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import derivatives as dv  # noqa: E402
from oracle import models as M  # noqa: E402
from oracle import mps as P  # noqa: E402


def fixture(name, L, terms, dtype, D, pos, seed):
    H = M.finite_mpo_hamiltonian(L, 2, terms, dtype=dtype)
    psi = P.finite_mps_from_tensors(P.random_initial_tensors(L, 2, D, seed, dtype))
    envs = P.FiniteEnvironments(psi, H)
    GL, GR = envs.leftenv(pos, psi), envs.rightenv(pos + 1, psi)
    rng = np.random.default_rng(seed + 1)
    shape = (GL.shape[0], 2, GR.shape[0], 2)
    x = rng.standard_normal(shape)
    if np.dtype(dtype).kind == "c":
        x = x + 1j * rng.standard_normal(shape)
    op = dv.JordanAC2(GL, H[pos], H[pos + 1], GR)
    y = op(x)
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), GL=GL, GR=GR, W1=H[pos],
                        W2=H[pos + 1], x=x, y=y, terms=np.array(",".join(op.terms())))
    print(name, op.terms(), np.linalg.norm(y))


def main():
    fixture("ac2_heisenberg_c128", 10, M.heisenberg_terms(10), np.complex128, 12, 4, 11)
    fixture("ac2_tfim_edge_f64", 8, M.tfim_terms(8, g=0.7, dtype=np.float64), np.float64, 8, 0, 12)
    fixture("ac2_j1j2_f64", 12, M.j1j2_cylinder_terms(4, 3), np.float64, 16, 5, 13)
    e = M.ed_ground_energy(10, 2, M.heisenberg_terms(10))[0]
    np.savez_compressed(os.path.join(HERE, "ed_heisenberg_L10.npz"), energy=e)
    print("ED L=10", e)


if __name__ == "__main__":
    main()
