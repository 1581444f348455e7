"""mpsgb -- GB300-native effective-Hamiltonian engine behind MPSKit.jl's derivative-operator API.

Host-side mirror of the MPSKit interface for the hot path (derivative operators, their
Krylov solvers, environment recursions and the DMRG drivers that call them); every
contraction runs in libmpsgb.so on the GPU.
"""
from . import _lib
from .core import Context, DeviceTensor, context
from .derivatives import (AC2_hamiltonian, AC_hamiltonian, C_hamiltonian, DerivativeOperator,
                          GB300Backend, Lanczos, MPO_AC2_Hamiltonian, MPO_AC_Hamiltonian,
                          exponentiate, fixedpoint, integrate, mpo_projection,
                          transfer_left, transfer_right)
from .operators import (FiniteMPOHamiltonian, InfiniteMPOHamiltonian, MPOHamiltonian,
                        heisenberg_XXX, j1j2_cylinder, transverse_field_ising, xxz)
from .states import (FiniteEnvironments, FiniteMPS, ac2_from, left_orth, mul_front, mul_tail,
                     project_complement_, right_orth, svd_trunc)
from .algorithms import (DMRG, DMRG2, DMRG3S, TDVP, AdaptiveKrylov, OptimalExpand,
                         SketchedExpand, changebonds, expectation_value, find_groundstate,
                         timestep, variance)
from .infinite import (IDMRG, VUMPS, InfiniteEnvironments, InfiniteMPS,
                       find_groundstate_idmrg, find_groundstate_vumps, timestep_infinite)
from .grassmann import GradientGrassmann
from . import optim
from . import u1
from . import batched
from . import io
from . import cell
from .cell import IDMRG2, InfiniteMPSCell, find_groundstate_idmrg2

__all__ = [
    "Context", "DeviceTensor", "context", "AC2_hamiltonian", "AC_hamiltonian", "C_hamiltonian",
    "DerivativeOperator", "GB300Backend", "Lanczos", "exponentiate", "fixedpoint", "integrate",
    "MPO_AC_Hamiltonian", "MPO_AC2_Hamiltonian", "mpo_projection", "transfer_left",
    "transfer_right",
    "FiniteMPOHamiltonian", "InfiniteMPOHamiltonian", "MPOHamiltonian", "heisenberg_XXX",
    "j1j2_cylinder", "transverse_field_ising", "xxz", "FiniteEnvironments", "FiniteMPS",
    "ac2_from", "left_orth", "mul_front", "mul_tail", "project_complement_", "right_orth",
    "svd_trunc", "DMRG", "DMRG2", "DMRG3S", "OptimalExpand", "SketchedExpand", "AdaptiveKrylov",
    "changebonds",
    "expectation_value", "find_groundstate", "variance", "GradientGrassmann", "optim",
    "TDVP", "timestep", "VUMPS", "IDMRG", "InfiniteEnvironments", "InfiniteMPS",
    "find_groundstate_vumps", "find_groundstate_idmrg", "timestep_infinite", "u1", "batched", "io",
    "cell", "IDMRG2", "InfiniteMPSCell", "find_groundstate_idmrg2",
]
