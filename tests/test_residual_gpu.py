"""GPU compensated residual (sfem_gb300_residual_dd) against the oracle's double-double
residual: the two evaluate b - A x of the same FP64 operator beyond FP64 accuracy, so
they agree to a few units of the residual's own rounding, not of |A||x|."""

import numpy as np
import pytest

import oracle as O
from sfem_gb300 import solvers as S
from sfem_gb300.mesh import SSMesh

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("kind", ["laplacian", "elasticity"])
def test_compensated_residual_matches_oracle(cuda, kind):
    import torch

    vec = 3 if kind == "elasticity" else 1
    m = SSMesh(4, 3, 2, 4, perturb=0.1, seed=5)
    H = S.Hierarchy(m, dirichlet_faces=("x0",), device=cuda, vec=vec)
    res = S.CompensatedResidual(H, kind, mu=1.0, lam=10.0)
    el = m.elements(4)
    n = vec * m.n_nodes()
    rng = np.random.default_rng(6)
    x = rng.standard_normal(n)
    dn = H.dirichlet[0].long().cpu().numpy()
    if kind == "laplacian":
        fff = H.fff.cpu().numpy().T.copy()
        ax = O.laplacian_residual_dd(4, el, fff, x, np.zeros(n))  # -A x, compensated
    else:
        adj, det = H.adj.cpu().numpy().T.copy(), H.det.cpu().numpy()
        ax = O.elasticity_residual_dd(4, el, adj, det, 1.0, 10.0, x, np.zeros(n))
    # b close to A x so the residual cancels almost completely
    b = -ax + 1e-9 * rng.standard_normal(n)
    rows = dn if vec == 1 else (vec * dn[:, None] + np.arange(vec)[None, :]).reshape(-1)
    if kind == "laplacian":
        ref = O.laplacian_residual_dd(4, el, fff, x, b)
    else:
        ref = O.elasticity_residual_dd(4, el, adj, det, 1.0, 10.0, x, b)
    ref[rows] = b[rows] - x[rows]
    got = res(torch.from_numpy(x).to(cuda), torch.from_numpy(b).to(cuda)).cpu().numpy()
    keep = np.ones(n, bool)
    keep[rows] = False
    # the residual entries are ~1e-9 while |A||x| is O(1): agreement to 1e-20 shows both
    # are far below the plain FP64 evaluation error (~1e-16)
    assert np.abs(got[keep] - ref[keep]).max() <= 1e-20 + 1e-12 * np.abs(ref[keep]).max()
    assert np.array_equal(got[rows], ref[rows])
