"""CPU restatement of the reference's solver templates (TEST INFRASTRUCTURE ONLY).

numpy loops over the oracle operators, following
  ConjugateGradient   algebra/sfem_cg.hpp:200-443 (plain and preconditioned)
  Chebyshev3          algebra/sfem_Chebyshev3.hpp:183-302
  PowerMethod         algebra/sfem_PowerMethod.hpp:18-55
  Multigrid::cycle    algebra/sfem_Multigrid.hpp:242-346
Used on small meshes only.
"""

from __future__ import annotations

import numpy as np


def cg(apply, b, x=None, precond=None, rtol=1e-10, atol=0.0, max_it=10000):
    """(P)CG; returns (x, iterations).  apply(v) returns A v."""
    x = np.zeros_like(b) if x is None else x.copy()
    r = b - apply(x)
    z = precond(r) if precond else r
    p = z.copy()
    rtz = float(r @ z)
    norm0 = np.sqrt(abs(rtz))
    if rtz == 0:
        return x, 0
    for it in range(1, max_it + 1):
        Ap = apply(p)
        alpha = rtz / float(p @ Ap)
        x += alpha * p
        r -= alpha * Ap
        z = precond(r) if precond else r
        rtz_new = float(r @ z)
        if np.sqrt(abs(rtz_new)) < atol or np.sqrt(abs(rtz_new)) / norm0 < rtol:
            return x, it
        p = z + (rtz_new / rtz) * p
        rtz = rtz_new
    return x, max_it


def random_uniform(n, seed):
    """U(-1, 1) from the splitmix64 hash of (seed, i), identical to sfem_gb300_random_uniform."""
    M = (1 << 64) - 1
    i = np.arange(1, n + 1, dtype=np.uint64)
    with np.errstate(over="ignore"):
        z = np.uint64(seed) + np.uint64(0x9E3779B97F4A7C15) * i
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    del M
    return (z >> np.uint64(11)).astype(np.float64) * (2.0 / 9007199254740992.0) - 1.0


def power_method(apply, n, max_it=100, tol=1e-5, v0=None):
    v = np.ones(n) if v0 is None else v0.copy()
    w = apply(v)
    w /= np.linalg.norm(w)
    vecs = [v, w]
    lam = lam_old = 0.0
    max_it_odd = max_it + (max_it % 2 == 0)
    for k in range(max_it_odd):
        wv = apply(vecs[(k + 1) % 2])
        lam = float(np.linalg.norm(wv))
        wv /= lam
        vecs[k % 2] = wv
        if abs(lam - lam_old) <= tol and k % 2 == 0:
            break
        lam_old = lam
    return lam


def chebyshev3(apply, b, x, eig_max, sweeps, scale_max=1.02, scale_min=0.06, inv_diag=None):
    """Chebyshev3; with inv_diag the iteration runs on D^-1 A (eig_max of D^-1 A)."""
    emax = eig_max * scale_max
    emin = scale_min * emax
    eavg, ediff = (emin + emax) / 2, (emin - emax) / 2
    alpha = 1.0 / eavg
    s = (lambda v: v) if inv_diag is None else (lambda v: inv_diag * v)
    p = s(apply(x) - b)
    x = x - alpha * p
    for it in range(1, sweeps):
        dea = ediff * alpha
        beta = (0.5 if it == 1 else 0.25) * dea * dea
        alpha = 1.0 / (eavg - beta / alpha)
        p = beta * p + s(apply(x) - b)
        x = x - alpha * p
    return x


def vcycle(levels, k, b, x):
    """levels[k] = dict(apply, smooth(b, x) -> x, restrict(r) -> rc, prolong(xc) -> xf, coarse_solve(b) -> x)."""
    L = levels[k]
    if k == len(levels) - 1:
        return L["coarse_solve"](b)
    x = L["smooth"](b, x)
    r = b - L["apply"](x)
    rc = L["restrict"](r)
    xc = vcycle(levels, k + 1, rc, np.zeros_like(rc))
    x = x + L["prolong"](xc)
    return L["smooth"](b, x)
