"""GradientGrassmann building blocks for finite MPS (oracle restatement, test infrastructure).

Restates src/algorithms/grassmann.jl for a FiniteMPS:
  * fg(state, H, envs)          -- grassmann.jl:150-169 (energy; per site
                                   Grassmann.project(AC_projection(i), AL[i]) * C[i]')
  * precondition(state, g)      -- grassmann.jl:73-91, rho_inv_regularized :243-255
  * retract(state, g, alpha)    -- grassmann.jl:93-108 (state'.AC[i] = (AL', C[i]) for all i,
                                   then normalize!: the AL' chain with the normalised last
                                   bond factor, orthoview.jl:152-183, finitemps.jl:627)
  * transport!(h, state, g, a, state')  -- grassmann.jl:124-136
  * inner(state, g1, g2)        -- grassmann.jl:61-71
The Grassmann tangent geometry of TensorKitManifolds (outside the reference sources) is
restated from Edelman, Arias & Smith, SIAM J. Matrix Anal. Appl. 20 (1998) 303-353,
eqs. (2.65) (geodesic) and (2.68) (parallel transport), with numpy's SVD.

Points are lists AL[0..L-1] (left-canonical, shape (Dl, d, Dr)) plus the 1 x 1 norm factor
of the last bond; tangents are lists of Z[i] with the same shapes.
"""
import numpy as np

from . import mps as P


def _mat(A):
    Dl, d, Dr = A.shape
    return A.reshape(Dl * d, Dr, order="F")


def _ten(M, shape):
    return M.reshape(shape, order="F")


def state_from_point(AL, Cend):
    """FiniteMPS of the point with AR and every C from the positive LQ sweep."""
    n = len(AL)
    C = [None] * (n + 1)
    C[n] = Cend
    psi = P.FiniteMPS([a.copy() for a in AL], [None] * n, C, n)
    return P.right_canonicalize(psi)


def fg(AL, Cend, H):
    """-> (energy, [Z_i]) at the point (AL, Cend)."""
    psi = state_from_point(AL, Cend)
    envs = P.FiniteEnvironments(psi, H)
    f = P.expectation_value(psi, H, envs, 0)
    gs = []
    for i in range(len(AL)):
        Ci = psi.C[i + 1]                       # MPSKit's C[i]: the bond right of site i
        AC = np.einsum("asb,bc->asc", AL[i], Ci)
        y = P.AC_hamiltonian(i, psi, H, envs)(AC)
        Y, W = _mat(y), _mat(AL[i])
        Z = Y - W @ (W.conj().T @ Y)            # Grassmann.project
        gs.append(_ten(Z @ Ci.conj().T, AL[i].shape))
    return float(f), gs


def rho_inv_regularized(C, rtol):
    U, S, _ = np.linalg.svd(C)
    d2 = (rtol * (S.max() if S.size else 0.0)) ** 2
    return (U * (1.0 / (S * S + d2))[None, :]) @ U.conj().T


def precondition(AL, Cend, g):
    psi = state_from_point(AL, Cend)
    rtolmin = np.finfo(np.float64).eps ** 0.75
    out = []
    for i, Z in enumerate(g):
        rtol = max(rtolmin, np.linalg.norm(Z))
        out.append(_ten(_mat(Z) @ rho_inv_regularized(psi.C[i + 1], rtol), Z.shape))
    return out


def _svd(Z):
    U, s, Vh = np.linalg.svd(_mat(Z), full_matrices=False)
    return U, s, Vh


def retract_site(W, Z, a):
    U, s, Vh = _svd(Z)
    Wm = _mat(W)
    WV = Wm @ Vh.conj().T
    Wn = Wm + (WV * (np.cos(a * s) - 1.0)[None, :] + U * np.sin(a * s)[None, :]) @ Vh
    # projectisometric: the polar factor (directions carry rounding noise off the tangent
    # space, most of all where the tangent space is empty and the preconditioner is large)
    Uw, _, Vw = np.linalg.svd(Wn, full_matrices=False)
    Wn = Uw @ Vw
    Zn = (-WV * (np.sin(a * s) * s)[None, :] + U * (np.cos(a * s) * s)[None, :]) @ Vh
    Zn = Zn - Wn @ (Wn.conj().T @ Zn)
    return _ten(Wn, W.shape), _ten(Zn, W.shape)


def retract(AL, Cend, g, a):
    res = [retract_site(W, Z, a) for W, Z in zip(AL, g)]
    return [r[0] for r in res], Cend / np.linalg.norm(Cend), [r[1] for r in res]


def transport_site(Th, W, Z, a, Wn):
    U, s, Vh = _svd(Z)
    Wm, Wnm, T = _mat(W), _mat(Wn), _mat(Th)
    WV = Wm @ Vh.conj().T
    M = -WV * np.sin(a * s)[None, :] + U * (np.cos(a * s) - 1.0)[None, :]
    out = T + M @ (U.conj().T @ T)
    out = out - Wnm @ (Wnm.conj().T @ out)
    return _ten(out, Th.shape)


def transport(h, AL, g, a, ALn):
    return [transport_site(h[i], AL[i], g[i], a, ALn[i]) for i in range(len(AL))]


def inner(g1, g2):
    return 2.0 * sum(np.real(np.vdot(a, b)) for a, b in zip(g1, g2))


# ---------------------------------------------------------------- one-site InfiniteMPS
def point_infinite(AL, C0):
    """InfiniteMPS(AL, C0) (infinitemps.jl:215-233): the right uniform gauge fixed from C0."""
    from . import vumps as V
    AR, C = V.uniform_rightorth(AL, C0)
    return V.InfiniteMPS1(AL, AR, C)


def fg_infinite(psi, W, chans):
    """fg(state::InfiniteMPS, H::InfiniteMPOHamiltonian) (grassmann.jl:171-190): fixed-point
    environments, energy density, Grassmann.project(AC_projection, AL) * C'."""
    from . import derivatives as dv
    from . import vumps as V
    GL, GR = V.infinite_envs(psi, W, chans, tol=1e-13)
    f = V.energy_density(psi, W, GL, GR)
    y = dv.JordanAC(GL, W, GR)(psi.AC)
    Y, A = _mat(y), _mat(psi.AL)
    Z = (Y - A @ (A.conj().T @ Y)) @ psi.C.conj().T
    return float(f), [_ten(Z, psi.AL.shape)]


def retract_infinite(psi, g, a):
    ALn, Zn = retract_site(psi.AL, g[0], a)
    return point_infinite(ALn, psi.C), [Zn]


def precondition_infinite(psi, g):
    rtol = max(np.finfo(np.float64).eps ** 0.75, np.linalg.norm(g[0]))
    return [_ten(_mat(g[0]) @ rho_inv_regularized(psi.C, rtol), g[0].shape)]


# ---------------------------------------------------------------- InfiniteMPS, L-site cell
def point_cell(AL, Cend):
    """InfiniteMPS(AL, C[end]) for a cell: AR and every C from the right uniform gauge."""
    from . import cell as Ce
    AR, C = Ce.uniform_rightorth(AL, Cend)
    return Ce.InfiniteMPSCell(AL, AR, C)


def fg_cell(psi, H):
    """fg(state::InfiniteMPS, H::InfiniteMPOHamiltonian) (grassmann.jl:171-190) for an L-site
    cell: the cell's fixed-point environments, the energy of the cell (expectation_value sums
    its sites, expval.jl:150-161) and per site Grassmann.project(AC_projection, AL[i]) C[i]'."""
    from . import cell as Ce
    from . import derivatives as dv
    GL, GR = Ce.infinite_envs(psi, H, tol=1e-13)
    f = Ce.energy(psi, H, GL, GR)
    gs = []
    for s in range(len(psi)):
        Y, A = _mat(dv.JordanAC(GL[s], H.W[s], GR[s])(psi.AC(s))), _mat(psi.AL[s])
        Z = (Y - A @ (A.conj().T @ Y)) @ psi.C[s].conj().T
        gs.append(_ten(Z, psi.AL[s].shape))
    return float(f), gs


def retract_cell(psi, g, a):
    """retract(state::InfiniteMPS, g, a) (grassmann.jl:106-115): every AL along its geodesic,
    then InfiniteMPS(AL', C[end])."""
    out = [retract_site(psi.AL[s], g[s], a) for s in range(len(psi))]
    return point_cell([o[0] for o in out], psi.C[-1]), [o[1] for o in out]


def transport_cell(h, psi, g, a, psin):
    return [transport_site(h[s], psi.AL[s], g[s], a, psin.AL[s]) for s in range(len(psi))]


def precondition_cell(psi, g):
    """precondition(state, g) (grassmann.jl:85-94): g[i] rho_inv_regularized(C[i])."""
    eps34 = np.finfo(np.float64).eps ** 0.75
    return [_ten(_mat(g[s]) @ rho_inv_regularized(psi.C[s], max(eps34, np.linalg.norm(g[s]))),
                 g[s].shape) for s in range(len(psi))]
