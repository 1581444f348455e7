"""Interchange format for MPOs, finite states and their environments: resume a run, or feed
an MPO built elsewhere (e.g. by the reference's channel-assignment builder,
src/operators/mpohamiltonian.jl:349-641, whose JordanMPOTensor blocks,
src/operators/jordanmpotensor.jl:44-137, embed densely as below).

One numpy ``.npz`` archive per object (readable from Julia with NPZ.jl).  Every tensor is a
dense block in the reference's (TensorKit) leg order, stored column-major:

  MPO    kind="mpo": finite (bool), nsites, W{i} = W[wl s; s' wr] with channel 0 = "not
         started" and channel wl-1 / wr-1 = "finished" (the sum space of a JordanMPOTensor:
         identity corners, C, B, A and D blocks), chans{i} (optional: dimensions of the
         channel blocks left of site i)
  state  kind="finite_mps": nsites, center, AL{i} = A[l s; r] for i < center, AR{i} for
         i >= center, C = C[l; r] of the centre bond, qb{i} (i = 0..nsites, bond charges)
         and qp (physical charges) for a U(1) state
  envs   kind="finite_envs": GL{i} = GL[a w; a'] and GR{i} = GR[b' w; b] for every
         environment held when saved

Loading a state uploads it; loading environments attaches them to a loaded state without
recomputation (they are taken as built from that state's AL / AR).
"""
import numpy as np

from . import _lib as L
from .core import DeviceTensor, PackedTensor, context
from .operators import MPOHamiltonian
from .states import FiniteEnvironments, FiniteMPS


def _f(a):
    return np.asfortranarray(a)


def save_mpo(path, H):
    out = {"kind": np.array("mpo"), "finite": np.array(bool(H.finite)),
           "nsites": np.array(len(H))}
    for i, w in enumerate(H.W):
        out[f"W{i}"] = _f(w)
    if H.chans is not None:
        for i, c in enumerate(H.chans):
            out[f"chans{i}"] = np.asarray(c, dtype=np.int64)
    np.savez(path, **out)


def load_mpo(path):
    with np.load(path) as z:
        if str(z["kind"]) != "mpo":
            raise ValueError(f"{path}: not an MPO archive")
        n = int(z["nsites"])
        W = [np.array(z[f"W{i}"]) for i in range(n)]
        chans = [np.array(z[f"chans{i}"]) for i in range(n)] if "chans0" in z else None
        for i in range(n):
            if W[i].ndim != 4 or W[i].shape[1] != W[i].shape[2]:
                raise ValueError(f"{path}: W{i} is not an MPO tensor W[wl s; s' wr]")
            if W[i].shape[3] != W[(i + 1) % n].shape[0] and (i + 1 < n or not bool(z["finite"])):
                raise ValueError(f"{path}: channel dimensions of sites {i} and {i + 1} differ")
        return MPOHamiltonian(W, finite=bool(z["finite"]), chans=chans)


def save_state(path, psi):
    """Download a device FiniteMPS into an archive."""
    n, c = len(psi), psi.center
    out = {"kind": np.array("finite_mps"), "nsites": np.array(n), "center": np.array(c),
           "C": _f(psi.C[c].numpy())}
    for i in range(n):
        if i < c:
            out[f"AL{i}"] = _f(psi.AL[i].numpy())
        else:
            out[f"AR{i}"] = _f(psi.AR[i].numpy())
    ch = psi.C[c].charges
    if ch is not None:
        ts = [psi.AL[i] if i < c else psi.AR[i] for i in range(n)]
        for i, t in enumerate(ts):
            out[f"qb{i}"] = np.asarray(t.charges[0], dtype=np.int32)
        out[f"qb{n}"] = np.asarray(ts[-1].charges[2], dtype=np.int32)
        out["qp"] = np.asarray(ts[0].charges[1], dtype=np.int32)
    np.savez(path, **out)


def load_state(path, ctx=None):
    """Upload an archived FiniteMPS (its centre and gauge as saved)."""
    ctx = ctx or context()
    with np.load(path) as z:
        if str(z["kind"]) != "finite_mps":
            raise ValueError(f"{path}: not a finite-MPS archive")
        n, c = int(z["nsites"]), int(z["center"])
        u1 = "qp" in z
        qb = [np.array(z[f"qb{i}"]) for i in range(n + 1)] if u1 else None
        qp = np.array(z["qp"]) if u1 else None
        AL, AR = [None] * n, [None] * n
        for i in range(n):
            key = f"AL{i}" if i < c else f"AR{i}"
            t = DeviceTensor.from_numpy(ctx, L.GB_KIND_MPS, np.array(z[key]))
            if u1:
                t.charges = (qb[i], qp, qb[i + 1])
            (AL if i < c else AR)[i] = t
        C = [None] * (n + 1)
        C[c] = DeviceTensor.from_numpy(ctx, L.GB_KIND_BOND, np.array(z["C"]))
        if u1:
            C[c].charges = (qb[c], qb[c])
    return FiniteMPS(AL, AR, C, c)


def save_environments(path, envs):
    out = {"kind": np.array("finite_envs"), "nsites": np.array(len(envs.GR) - 1)}
    host = lambda g: _f((g.unpack() if isinstance(g, PackedTensor) else g).numpy())
    for i, g in enumerate(envs.GL):
        if g is not None:
            out[f"GL{i}"] = host(g)
    for i, g in enumerate(envs.GR):
        if g is not None:
            out[f"GR{i}"] = host(g)
    np.savez(path, **out)


def load_environments(path, psi, H, ctx=None):
    """FiniteEnvironments of `psi` with the archived GL / GR attached: GL[i] counts as built
    from psi.AL[0..i-1] and GR[i] from psi.AR[i+1..], so nothing is recomputed."""
    ctx = ctx or psi.ctx
    envs = FiniteEnvironments(psi, H, ctx)
    n = len(psi)
    with np.load(path) as z:
        if str(z["kind"]) != "finite_envs" or int(z["nsites"]) != n:
            raise ValueError(f"{path}: not the environments of a {n}-site state")
        for i in range(n + 1):
            if f"GL{i}" in z:
                envs.GL[i] = DeviceTensor.from_numpy(ctx, L.GB_KIND_GL,
                                                     np.array(z[f"GL{i}"]), envs.dtype)
                for j in range(i):
                    envs.ldep[j] = psi.AL[j]
            if f"GR{i}" in z:
                envs.GR[i] = DeviceTensor.from_numpy(ctx, L.GB_KIND_GR,
                                                     np.array(z[f"GR{i}"]), envs.dtype)
                for j in range(i + 1, n):
                    envs.rdep[j] = psi.AR[j]
    return envs
