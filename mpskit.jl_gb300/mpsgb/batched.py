"""Many independent chains solved at once (a coupling sweep).

MPSKit solves independent problems one after another (or from separate Julia tasks, each
calling the derivative constructors; src/algorithms/groundstate/vumps.jl:142-151).  Here each
instance runs its whole VUMPS loop on one of `workers` contexts -- every context owns a CUDA
stream, its scratch buffers and its cuSOLVER handle -- driven by a pool of host threads.  The
library releases the Python GIL inside every call, so the kernels of different instances
reach the GPU from concurrent streams: at the small bond dimensions of a coupling sweep
(D = 64..256) one instance's GEMMs occupy a handful of SMs and the other streams fill the
rest.  Results are identical to solving the instances one by one (every kernel is
deterministic per instance).
"""
import concurrent.futures as cf
import queue
import threading
import time

import numpy as np

from . import _lib as L
from .core import Context
from .infinite import (VUMPS, InfiniteEnvironments, InfiniteMPS, energy_density,
                       find_groundstate_vumps)
from .operators import transverse_field_ising


class Instance:
    """One chain of the sweep: its Hamiltonian, initial tensor and (after solving) result."""

    def __init__(self, H, A0, label=None):
        self.H, self.A0, self.label = H, A0, label
        self.energy = None
        self.energy_split = None  # energy of the split-precision environments, if any
        self.eps = None
        self.iterations = 0
        self.seconds = 0.0
        self.history = None


def tfim_sweep(n=64, gmin=0.1, gmax=2.0, dims=(64, 128, 192, 256), seed=1234 + 4, J=1.0,
               dtype=np.complex128):
    """n transverse-field Ising chains (-J sum Z Z - g sum X), g uniformly spaced in
    [gmin, gmax], bond dimension drawn from `dims` by seed, i.i.d. normal initial tensors."""
    rng = np.random.default_rng(seed)
    out = []
    for g in np.linspace(gmin, gmax, n):
        D = int(rng.choice(dims))
        shape = (D, 2, D)
        if np.dtype(dtype).kind == "c":
            A0 = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
        else:
            A0 = rng.standard_normal(shape)
        H = transverse_field_ising(1, g=float(g), J=J, dtype=dtype, infinite=True)
        out.append(Instance(H, np.asarray(A0, dtype=dtype), label={"g": float(g), "D": D}))
    return out


def solve_vumps_batched(instances, alg=None, workers=16, device=0, contexts=None):
    """find_groundstate(InfiniteMPS, H, VUMPS()) for every instance, `workers` at a time.
    Returns the instances with energy, eps, iterations and seconds filled in."""
    alg = alg or VUMPS()
    ctxs = contexts or [Context(device) for _ in range(max(1, workers))]
    pool = queue.Queue()
    for c in ctxs:
        pool.put(c)
    errors = []
    lock = threading.Lock()

    def run(inst):
        ctx = pool.get()
        try:
            t0 = time.perf_counter()
            psi = InfiniteMPS.from_tensor(inst.A0, ctx)
            psi, envs, eps, hist = find_groundstate_vumps(psi, inst.H, alg)
            inst.energy = hist[-1]["energy"] if hist else None
            if alg.backend.code != L.GB_PREC_FP64:
                # the FP64 refinement step: energy density from FP64 environments of the
                # converged state (the split-precision environments carry the contraction
                # error to first order)
                inst.energy_split = inst.energy
                env64 = InfiniteEnvironments(psi, inst.H, L.GB_PREC_FP64)
                env64.recalculate(psi, tol=1e-12)
                inst.energy = energy_density(psi, env64)
            ctx.synchronize()
            inst.seconds = time.perf_counter() - t0
            inst.eps = eps
            inst.iterations = len(hist)
            inst.history = hist
        except Exception as e:  # reported after the pool drains
            with lock:
                errors.append((inst.label, e))
        finally:
            pool.put(ctx)

    # largest instances first: the tail of the sweep is then made of short jobs
    order = sorted(instances, key=lambda i: -i.A0.shape[0])
    with cf.ThreadPoolExecutor(max_workers=len(ctxs)) as ex:
        list(ex.map(run, order))
    if errors:
        label, e = errors[0]
        raise RuntimeError(f"instance {label} failed: {e}") from e
    return instances
