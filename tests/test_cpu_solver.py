"""CPU oracle solver and compensated residuals (test infrastructure checks).

* or_mg_pcg_solve (oracle/src/solve.c), the restated reference CG + V-cycle +
  Chebyshev3, reaches a true residual of 1e-10 on small Poisson and cantilever problems
  and agrees with the numpy restatement's plain CG solution;
* the double-double residuals agree with the plain FP64 residual where that one is
  accurate, and stay accurate where it is not (a right-hand side built as A x exactly).
"""

import numpy as np
import pytest

import oracle as O
from sfem_gb300.mesh import SSMesh


def _lumped_force(m, det):
    L = m.L
    el = m.elements(L)
    N1 = L + 1
    lid = np.arange(N1 ** 3)
    xi, yi, zi = lid % N1, (lid // N1) % N1, lid // (N1 * N1)
    mult = np.ones(N1 ** 3)
    for c in (xi, yi, zi):
        mult *= np.where((c == 0) | (c == L), 1.0, 2.0)
    w = mult[:, None] * (det.astype(np.float64) / (8.0 * L ** 3))[None, :]
    vol = np.bincount(el.reshape(-1), weights=w.reshape(-1), minlength=m.n_nodes())
    b = np.zeros(3 * m.n_nodes())
    b[2::3] = -vol
    return b


def test_cpu_mg_pcg_poisson_matches_plain_cg():
    m = SSMesh(4, 4, 3, 4, perturb=0.1, seed=1)
    el = m.elements(4)
    fff = O.fff_fill(el[m.macro_corner_lidx(4)], m.points)
    dn = m.boundary_nodes("x0", 4)
    b = np.random.default_rng(2).standard_normal(m.n_nodes())
    b[dn] = 0
    x, st = O.mg_pcg_solve(m, "laplacian", b, geom=fff, flexible=True)
    assert st["rc"] == 0 and st["true_rel_residual"] <= 1e-10 and st["iterations"] < 30

    def A(v):
        y = O.sshex8_laplacian_stencil_apply(4, el, fff, v)
        y[dn] = v[dn]
        return y

    import oracle.solvers as OS

    xr, _ = OS.cg(A, b, rtol=1e-13, max_it=5000)
    assert np.linalg.norm(x - xr) <= 1e-8 * np.linalg.norm(xr)


def test_cpu_mg_pcg_cantilever():
    m = SSMesh(8, 2, 2, 4, box=((0, 4), (0, 1), (0, 1)), perturb=0.0, seed=0)
    el = m.elements(4)
    adj, det = O.adjugate_fill(el[m.macro_corner_lidx(4)], m.points)
    b = _lumped_force(m, det)
    dn = m.boundary_nodes("x0", 4)
    for c in range(3):
        b[3 * dn + c] = 0
    x, st = O.mg_pcg_solve(m, "elasticity", b, geom=adj, det=det, scale_eig_max=1.1, coarse_rtol=1e-6,
                           flexible=True, max_it=300)
    assert st["rc"] == 0 and st["true_rel_residual"] <= 1e-10
    r = O.elasticity_residual_dd(4, el, adj, det, 1.0, 10.0, x, b)
    for c in range(3):
        r[3 * dn + c] = b[3 * dn + c] - x[3 * dn + c]
    assert np.linalg.norm(r) <= 1.5e-10 * np.linalg.norm(b)


@pytest.mark.parametrize("kind", ["laplacian", "elasticity"])
def test_double_double_residual(kind):
    """On random data the compensated residual equals the FP64 one to FP64 rounding;
    for b = A x formed in double-double from a random x it is ~0 while the plain FP64
    residual keeps its rounding error."""
    m = SSMesh(3, 2, 2, 4, perturb=0.1, seed=3)
    el = m.elements(4)
    corners = el[m.macro_corner_lidx(4)]
    rng = np.random.default_rng(4)
    if kind == "laplacian":
        fff = O.fff_fill(corners, m.points)
        n = m.n_nodes()
        apply = lambda v: O.sshex8_laplacian_stencil_apply(4, el, fff, v)
        resid = lambda v, b: O.laplacian_residual_dd(4, el, fff, v, b)
    else:
        adj, det = O.adjugate_fill(corners, m.points)
        n = 3 * m.n_nodes()
        apply = lambda v: O.linear_elasticity_apply(4, el, adj, det, 1.0, 10.0, v)
        resid = lambda v, b: O.elasticity_residual_dd(4, el, adj, det, 1.0, 10.0, v, b)
    x, b = rng.standard_normal(n), rng.standard_normal(n)
    scale = np.abs(apply(np.abs(x))).max() + np.abs(b).max()
    assert np.abs(resid(x, b) - (b - apply(x))).max() <= 1e-14 * scale
    # b = A x carried beyond double: (hi, lo) with b_hi = fl(A x); the residual of x against
    # b_hi is then b_hi - A x = -(rounding of A x), far below the plain evaluation error
    bh = -resid(x, np.zeros(n))  # A x, compensated, rounded once
    r = resid(x, bh)
    assert np.abs(r).max() <= 2 * np.spacing(np.abs(bh)).max()
