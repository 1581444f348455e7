"""Derivative operators and their Krylov solvers (host mirror of MPSKit's API).

  AC2_hamiltonian / AC_hamiltonian / C_hamiltonian
      -- src/algorithms/derivatives/hamiltonian_derivatives.jl:44-55, 206-217,
         src/algorithms/derivatives/mpo_derivatives.jl:37-45
  MPO_AC_Hamiltonian / MPO_AC2_Hamiltonian (an arbitrary MPO, no Jordan structure)
      -- src/algorithms/derivatives/mpo_derivatives.jl:46-66
  mpo_projection (C/AC/AC2_projection between different bra and ket states)
      -- src/algorithms/derivatives/derivatives.jl:194-216
  transfer_left / transfer_right (one environment step, bra and ket given separately)
      -- src/algorithms/toolbox/transfer.jl:125-130 (also src/environments/finite_envs.jl)
  fixedpoint(H, x0, :SR, Lanczos)       -- src/algorithms/fixedpoint.jl:15-18
  integrate(H, y0, t, dt, Lanczos)      -- src/algorithms/timestep/integrators.jl:44-53

Every operator is a handle to a prepared operator living on the GPU; applying it and
solving with it run entirely on the device through libmpsgb.
"""
import ctypes
from dataclasses import dataclass

import numpy as np

from . import _lib as L
from .core import DeviceTensor


@dataclass
class GB300Backend:
    """Contraction backend selecting the GB300 engine (the `backend` seam of
    DMRG/DMRG2/VUMPS/TDVP, src/algorithms/groundstate/dmrg.jl:86-87).

    precision: "fp64" (plain), "bf16x3" or "tf32x3" (split-precision tensor-core
    contractions with BF16 or TF32 hi/lo operands, FP64 Krylov/gauge steps)."""
    precision: str = "fp64"
    device: int = 0

    @property
    def code(self):
        return L.PRECISIONS[self.precision]


@dataclass
class Lanczos:
    """KrylovKit.Lanczos parameters used by MPSKit's eigensolves."""
    krylovdim: int = 30
    maxiter: int = 100
    tol: float = 1e-12
    eager: bool = False


class DerivativeOperator:
    """A prepared effective Hamiltonian (C, AC or AC2) on the device."""

    def __init__(self, ctx, kind, GL, W1, W2, GR, backend):
        self.ctx = ctx
        # the generic-MPO kinds act as the Jordan kinds of the same arity
        self.kind = {L.GB_HEFF_AC_MPO: L.GB_HEFF_AC, L.GB_HEFF_AC2_MPO: L.GB_HEFF_AC2}.get(kind, kind)
        self.generic = kind in (L.GB_HEFF_AC_MPO, L.GB_HEFF_AC2_MPO)
        self.backend = backend
        h = ctypes.c_void_p()
        L.check(L.lib().gb_heff_build(ctx.handle, kind, GL.handle,
                                      W1.handle if W1 is not None else None,
                                      W2.handle if W2 is not None else None,
                                      GR.handle, backend.code, ctypes.byref(h)))
        self.handle = h
        # keep the environments alive: the operator references their device storage
        self._keep = (GL, GR, W1, W2)
        self._sectors = None
        self.dtype = GL.dtype
        Dl, Dr = GL.dims[0], GR.dims[0]
        if self.kind == L.GB_HEFF_AC2:
            self.xkind, self.xdims = L.GB_KIND_AC2, (Dl, W1.dims[1], Dr, W2.dims[1])
        elif self.kind == L.GB_HEFF_AC:
            self.xkind, self.xdims = L.GB_KIND_MPS, (Dl, W1.dims[1], Dr)
        else:
            self.xkind, self.xdims = L.GB_KIND_BOND, (Dl, Dr)

    @property
    def terms(self):
        buf = ctypes.create_string_buffer(256)
        L.check(L.lib().gb_heff_terms(self.handle, buf, 256))
        return tuple(t for t in buf.value.decode().split(",") if t)

    def describe(self):
        """Per-step contraction shapes and grouped sector-block plans (gb_heff_describe)."""
        buf = ctypes.create_string_buffer(1 << 16)
        L.check(L.lib().gb_heff_describe(self.handle, buf, 1 << 16))
        return buf.value.decode()

    @property
    def flops(self):
        v = ctypes.c_double()
        L.check(L.lib().gb_heff_flops(self.handle, ctypes.byref(v)))
        return v.value

    def set_precision(self, precision):
        code = L.PRECISIONS[precision]
        L.check(L.lib().gb_heff_set_precision(self.handle, code))

    def set_sectors(self, x):
        """Hand the U(1) leg charges of x (AC: (l, s, r); AC2: (l, s1, r, s2)) to the
        operator once (gb_heff_set_sectors): its fused chain then skips the exact zeros of
        the charge-sorted embedding.  No-op for dense vectors and C operators."""
        if self._sectors is not None or x.charges is None or self.kind == L.GB_HEFF_C:
            return
        q = [np.ascontiguousarray(c, dtype=np.int32) for c in x.charges]
        p = lambda a: a.ctypes.data_as(L.PI32)
        if self.kind == L.GB_HEFF_AC2:
            ql, qs1, qr, qs2 = q
            L.check(L.lib().gb_heff_set_sectors(self.handle, p(ql), p(qs1), p(qs2), p(qr)))
        else:
            ql, qs, qr = q
            L.check(L.lib().gb_heff_set_sectors(self.handle, p(ql), p(qs), None, p(qr)))
        self._sectors = q

    def new_vector(self):
        return DeviceTensor(self.ctx, self.xkind, self.dtype, self.xdims)

    def __call__(self, x, out=None):
        self.set_sectors(x)
        y = out if out is not None else x.similar()
        L.check(L.lib().gb_heff_apply(self.handle, x.handle, y.handle))
        return y

    __mul__ = __call__

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and L._lib is not None:
            try:
                L.lib().gb_heff_free(h)
            except Exception:
                pass
            self.handle = None


def AC2_hamiltonian(site, psi, H, envs, backend=None):
    """JordanMPO_AC2_Hamiltonian for bond (site, site+1), prepared."""
    backend = backend or GB300Backend()
    ctx = envs.ctx
    W = H.device(ctx, envs.dtype)
    return DerivativeOperator(ctx, L.GB_HEFF_AC2, envs.leftenv(site, psi), W[site], W[site + 1],
                              envs.rightenv(site + 1, psi), backend)


def AC_hamiltonian(site, psi, H, envs, backend=None):
    backend = backend or GB300Backend()
    ctx = envs.ctx
    W = H.device(ctx, envs.dtype)
    return DerivativeOperator(ctx, L.GB_HEFF_AC, envs.leftenv(site, psi), W[site], None,
                              envs.rightenv(site, psi), backend)


def MPO_AC_Hamiltonian(GL, W, GR, backend=None):
    """MPO_AC_Hamiltonian(GL, W, GR) of an arbitrary MPO tensor (mpo_derivatives.jl:46-55,
    100-107): y = GL . x . W . GR over every channel pair."""
    return DerivativeOperator(GL.ctx, L.GB_HEFF_AC_MPO, GL, W, None, GR,
                              backend or GB300Backend())


def MPO_AC2_Hamiltonian(GL, W1, W2, GR, backend=None):
    """MPO_AC2_Hamiltonian(GL, W1, W2, GR) of an arbitrary MPO (mpo_derivatives.jl:56-66,
    144-153)."""
    return DerivativeOperator(GL.ctx, L.GB_HEFF_AC2_MPO, GL, W1, W2, GR,
                              backend or GB300Backend())


def _fuse_two_site(W1, W2):
    """W1 W2 over their shared channel as one MPO tensor (wl, d1 d2, d1 d2, wr), physical
    index s1 + d1 s2 (the device order of a two-site tensor's physical legs)."""
    wl, d1, _, _ = W1.shape
    _, d2, _, wr = W2.shape
    W = np.einsum("asum,mtvb->astuvb", W1, W2)  # (wl, s1, s2, t1, t2, wr)
    return np.asfortranarray(W.reshape(wl, d1 * d2, d1 * d2, wr, order="F"))


def _mpo_tensor(ctx, W):
    return W if isinstance(W, DeviceTensor) else DeviceTensor.from_numpy(ctx, L.GB_KIND_MPO,
                                                                          np.asarray(W))


def mpo_projection(GL, GR, x, W1=None, W2=None, backend=None):
    """One application of a generic derivative operator between different bra and ket states
    (C_projection / AC_projection / AC2_projection with below != above,
    derivatives.jl:194-216, through MPO_C/AC/AC2_Hamiltonian, mpo_derivatives.jl:37-66):
    GL[bra l w; ket l'], GR[ket r' w; bra r]; W1 a device MPO tensor or a host array
    (wl, d, d, wr) (W1 and W2 host arrays for the two-site form), or None for the bond
    operator.  Returns y on the bra bonds (gb_mpo_project)."""
    backend = backend or GB300Backend()
    ctx = x.ctx
    Dlb, Drb = GL.dims[0], GR.dims[2]
    if W1 is None:
        y = DeviceTensor(ctx, L.GB_KIND_BOND, x.dtype, (Dlb, Drb))
        L.check(L.lib().gb_mpo_project(ctx.handle, GL.handle, None, GR.handle, x.handle,
                                       backend.code, y.handle))
        return y
    if W2 is None:
        W = _mpo_tensor(ctx, W1)
        y = DeviceTensor(ctx, L.GB_KIND_MPS, x.dtype, (Dlb, W.dims[1], Drb))
        L.check(L.lib().gb_mpo_project(ctx.handle, GL.handle, W.handle, GR.handle, x.handle,
                                       backend.code, y.handle))
        return y
    d1, d2 = W1.shape[1], W2.shape[1]
    W = DeviceTensor.from_numpy(ctx, L.GB_KIND_MPO, _fuse_two_site(np.asarray(W1), np.asarray(W2)))
    xf = x.copy().reshape_(L.GB_KIND_MPS, (x.dims[0], d1 * d2, x.dims[2]))
    y = DeviceTensor(ctx, L.GB_KIND_MPS, x.dtype, (Dlb, d1 * d2, Drb))
    L.check(L.lib().gb_mpo_project(ctx.handle, GL.handle, W.handle, GR.handle, xf.handle,
                                   backend.code, y.handle))
    return y.reshape_(L.GB_KIND_AC2, (Dlb, d1, Drb, d2))


def transfer_left(GL, W, A, Abar=None, backend=None):
    """transfer_left(GL, O, A, Abar) (transfer.jl:125-127): GL'[a w'; a'] =
    GL[b w; b'] A[b' s'; a'] W[w s; s' w'] conj(Abar[b s; a]); Abar defaults to A.  W is a
    device MPO tensor or a host array (wl, d, d, wr).  Runs gb_env_transfer_left."""
    backend = backend or GB300Backend()
    ctx = A.ctx
    Abar = A if Abar is None else Abar
    Wd = _mpo_tensor(ctx, W)
    out = DeviceTensor(ctx, L.GB_KIND_GL, GL.dtype, (Abar.dims[2], Wd.dims[3], A.dims[2]))
    L.check(L.lib().gb_env_transfer_left(ctx.handle, GL.handle, Wd.handle, A.handle, Abar.handle,
                                         backend.code, out.handle))
    return out


def transfer_right(GR, W, A, Abar=None, backend=None):
    """transfer_right(GR, O, A, Abar) (transfer.jl:128-130): GR'[a' w; a] =
    A[a' s'; b'] W[w s; s' w'] GR[b' w'; b] conj(Abar[a s; b]); Abar defaults to A.
    Runs gb_env_transfer_right."""
    backend = backend or GB300Backend()
    ctx = A.ctx
    Abar = A if Abar is None else Abar
    Wd = _mpo_tensor(ctx, W)
    out = DeviceTensor(ctx, L.GB_KIND_GR, GR.dtype, (A.dims[0], Wd.dims[0], Abar.dims[0]))
    L.check(L.lib().gb_env_transfer_right(ctx.handle, GR.handle, Wd.handle, A.handle, Abar.handle,
                                          backend.code, out.handle))
    return out


def C_hamiltonian(site, psi, H, envs, backend=None):
    """MPO_C_Hamiltonian of the bond right of `site` (GL[site+1], GR[site])."""
    backend = backend or GB300Backend()
    return DerivativeOperator(envs.ctx, L.GB_HEFF_C, envs.leftenv(site + 1, psi), None, None,
                              envs.rightenv(site, psi), backend)


class Info:
    def __init__(self, ki):
        self.converged = ki.converged
        self.numops = ki.numops
        self.numiter = ki.numiter
        self.normres = ki.normres

    def __repr__(self):
        return (f"Info(converged={self.converged}, normres={self.normres:.3e}, "
                f"numops={self.numops}, numiter={self.numiter})")


def fixedpoint(A, x0, which="SR", alg=None):
    """Lowest eigenpair (val, vec, info); x0 is not modified."""
    if which != "SR":
        raise NotImplementedError("only :SR eigensolves run on the device")
    alg = alg or Lanczos()
    A.set_sectors(x0)
    x = x0.copy()
    lam = ctypes.c_double()
    ki = L.KrylovInfo()
    L.check(L.lib().gb_heff_eigsolve(A.handle, x.handle, int(alg.krylovdim), int(alg.maxiter),
                                     float(alg.tol), int(bool(alg.eager)), ctypes.byref(lam),
                                     ctypes.byref(ki)))
    return lam.value, x, Info(ki)


def exponentiate(A, t, x0, alg=None):
    """exp(t A) x0 (KrylovKit.exponentiate); returns (y, info)."""
    alg = alg or Lanczos(tol=1e-12)
    A.set_sectors(x0)
    t = complex(t)
    y = x0.copy()
    ki = L.KrylovInfo()
    L.check(L.lib().gb_heff_exponentiate(A.handle, y.handle, t.real, t.imag, int(alg.krylovdim),
                                         int(alg.maxiter), float(alg.tol), ctypes.byref(ki)))
    return y, Info(ki)


def integrate(A, y0, t, dt, alg=None, imaginary_evolution=False):
    """integrate(f, y0, t, dt, alg) for a time-independent operator
    (integrators.jl:44-53): exp(-i dt A) y0, or exp(-dt A) y0 in imaginary time."""
    tt = -dt if imaginary_evolution else -1j * dt
    y, info = exponentiate(A, tt, y0, alg)
    if info.converged == 0:
        import warnings
        warnings.warn(f"integrator failed to converge: {info}")
    return y
