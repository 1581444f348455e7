"""Riemannian conjugate-gradient optimisation: the `method` of GradientGrassmann
(src/algorithms/groundstate/gradient_grassmann.jl:47-78, 80-121).  The reference delegates to
OptimKit.jl (compat 0.4, 0.5 in Project.toml), a dependency outside the reference sources:
`optimize(fg, x, ConjugateGradient(; gradtol, maxiter, linesearch = HagerZhangLineSearch()))`
with user retract / transport! / inner / precondition callbacks.  This module restates the
published methods OptimKit implements, on the same callback interface:

  * nonlinear CG with the Hager-Zhang direction update (W. W. Hager, H. Zhang, "A new
    conjugate gradient method with guaranteed descent and an efficient line search",
    SIAM J. Optim. 16 (2005) 170-192; preconditioned form and the eta lower bound as in
    Hager & Zhang, "The limited memory conjugate gradient method", SIAM J. Optim. 23 (2013)
    2150-2168), on a manifold by transporting the previous gradient and direction;
  * the line search of the same papers (CG_DESCENT, ACM TOMS 32 (2006) 113-137): bracketing,
    the double secant step and bisection, accepting the Wolfe or the approximate Wolfe
    conditions.

Everything here is host logic over opaque points and tangent vectors; the vector operations
are the callbacks (for GradientGrassmann they run on the device).
"""
import math
from dataclasses import dataclass, field


@dataclass
class HagerZhangLineSearch:
    """Line search with the (approximate) Wolfe conditions of Hager & Zhang.
    delta, sigma: Wolfe constants; epsilon: relative slack of the approximate conditions;
    theta: bisection weight; gamma: required interval shrink per secant pass; rho: bracket
    expansion factor; maxiter: bound on function evaluations."""
    delta: float = 0.1
    sigma: float = 0.9
    epsilon: float = 1e-6
    theta: float = 0.5
    gamma: float = 2.0 / 3.0
    rho: float = 5.0
    maxiter: int = 100

    def __call__(self, fg, x0, eta, f0, g0, alpha0, retract, inner):
        """-> (x, f, g, xi, alpha, nfg): the accepted point, its value and gradient, the
        direction transported to it (from retract) and the step."""
        dphi0 = inner(x0, g0, eta)
        if not dphi0 < 0:
            raise ValueError(f"line search: not a descent direction (slope {dphi0})")
        fmax = f0 + self.epsilon * abs(f0)
        state = {"n": 0, "best": None}

        class _Accepted(Exception):
            pass

        def take(c):
            if state["n"] >= self.maxiter:
                raise _Accepted()
            state["n"] += 1
            x, xi = retract(x0, eta, c)
            f, g = fg(x)
            p = _Point(c, x, f, g, xi, inner(x, g, xi))
            if math.isfinite(p.f) and p.f <= fmax and (state["best"] is None
                                                       or p.f < state["best"].f):
                state["best"] = p
            wolfe = p.f - f0 <= self.delta * c * dphi0 and p.dphi >= self.sigma * dphi0
            approx = ((2 * self.delta - 1) * dphi0 >= p.dphi >= self.sigma * dphi0
                      and p.f <= fmax)
            if wolfe or approx:
                state["hit"] = p
                raise _Accepted()
            return p

        def u3(a, b):
            # shrink [a, b] (a: slope < 0 and f <= fmax) by weighted bisection
            while True:
                p = take((1 - self.theta) * a.c + self.theta * b.c)
                if p.dphi >= 0:
                    return a, p
                if p.f <= fmax:
                    a = p
                else:
                    b = p

        def update(a, b, c):
            if not a.c < c < b.c:
                return a, b, None
            p = take(c)
            if p.dphi >= 0:
                return a, p, p
            if p.f <= fmax:
                return p, b, p
            a2, b2 = u3(a, p)
            return a2, b2, p

        def secant(a, b):
            den = b.dphi - a.dphi
            if den == 0 or not math.isfinite(den):
                return math.nan
            return (a.c * b.dphi - b.c * a.dphi) / den

        p0 = _Point(0.0, x0, f0, g0, eta, dphi0)
        try:
            # bracket
            a, c = p0, alpha0
            while True:
                p = take(c)
                if p.dphi >= 0:
                    b = p
                    break
                if p.f > fmax:
                    a, b = u3(p0, p)
                    break
                a, c = p, self.rho * c
            # secant^2 / bisection passes
            while True:
                width = b.c - a.c
                A, B, pc = update(a, b, secant(a, b))
                if pc is not None and (pc is A or pc is B):
                    cbar = secant(b, B) if pc is B else secant(a, A)
                    A, B, _ = update(A, B, cbar)
                if B.c - A.c > self.gamma * width:
                    A, B, _ = update(A, B, 0.5 * (A.c + B.c))
                a, b = A, B
                if b.c - a.c <= 1e-14 * max(b.c, 1e-300):
                    raise _Accepted()
        except _Accepted:
            p = state.get("hit") or state["best"]
            if p is None:
                raise RuntimeError("line search: no acceptable step found")
        return p.x, p.f, p.g, p.xi, p.c, state["n"]


@dataclass
class _Point:
    c: float
    x: object
    f: float
    g: object
    xi: object
    dphi: float


@dataclass
class ConjugateGradient:
    """ConjugateGradient(; gradtol, maxiter, linesearch) with the Hager-Zhang update:
    beta = (<y, Pg> - theta <y, Py> <d, g> / <d, y>) / <d, y>, bounded below by
    eta <d, g_prev> / <d, d>; restart (beta = 0) every `restart` iterations."""
    gradtol: float = 1e-8
    maxiter: int = 200
    linesearch: HagerZhangLineSearch = field(default_factory=HagerZhangLineSearch)
    eta: float = 0.4
    theta: float = 1.0
    restart: int = 1 << 30
    verbosity: int = 0


def optimize(fg, x, alg, retract, transport, inner, add, scale, precondition=None,
             hasconverged=None, shouldstop=None, finalize=None):
    """optimize(fg, x, alg; retract, transport!, inner, add!, scale!, precondition) ->
    (x, f, g, numfg, normgradhistory).

    fg(x) -> (f, g);  retract(x, d, a) -> (x', d transported to x');
    transport(v, x, d, a, x') -> v at x';  inner(x, v, w) -> real;
    add(v, w, a, b) -> a v + b w (new);  scale(v, a) -> a v (new);
    precondition(x, g) -> P g (new; identity when None)."""
    precondition = precondition or (lambda x_, g_: scale(g_, 1.0))
    hasconverged = hasconverged or (lambda x_, f_, g_, ng: ng <= alg.gradtol)
    shouldstop = shouldstop or (lambda x_, f_, g_, nfg, it: it >= alg.maxiter)
    f, g = fg(x)
    numfg = 1
    ng = math.sqrt(max(inner(x, g, g), 0.0))
    history = [ng]
    Pg = precondition(x, g)
    d = scale(Pg, -1.0)
    alpha = 1.0
    it = 0
    while not (hasconverged(x, f, g, ng) or shouldstop(x, f, g, numfg, it)):
        if inner(x, d, g) >= 0:  # lost descent: restart along -Pg
            d = scale(Pg, -1.0)
        xp, gp, Pgp = x, g, Pg
        x, f, g, xi, alpha, nfg = alg.linesearch(fg, xp, d, f, gp, alpha, retract, inner)
        numfg += nfg
        it += 1
        if finalize is not None:
            x, f, g = finalize(x, f, g, it)
        ng = math.sqrt(max(inner(x, g, g), 0.0))
        history.append(ng)
        if alg.verbosity > 0:
            print(f"CG: iter {it:4d}: f = {f:.12f}, |g| = {ng:.4e}, step {alpha:.3e}, "
                  f"{nfg} evaluations")
        if hasconverged(x, f, g, ng):
            break
        Pg = precondition(x, g)
        gpt = transport(gp, xp, d, alpha, x)
        Pgpt = transport(Pgp, xp, d, alpha, x)
        dt = xi
        y = add(g, gpt, 1.0, -1.0)
        Py = add(Pg, Pgpt, 1.0, -1.0)
        dy = inner(x, dt, y)
        beta = 0.0
        if dy != 0 and it % alg.restart != 0:
            beta = (inner(x, y, Pg) - alg.theta * inner(x, y, Py) * inner(x, dt, g) / dy) / dy
            dd = inner(x, dt, dt)
            if dd > 0:
                beta = max(beta, alg.eta * inner(x, dt, gpt) / dd)
        d = add(Pg, dt, -1.0, beta)
    return x, f, g, numfg, history
