"""GPU compensated residual (sfem_gb300_residual_dd) against the oracle's double-double
residual evaluated from the same micro element matrices: both give b - A x of one FP64
operator beyond FP64 accuracy, so they agree to the rounding of the residual itself,
far below the ~1e-16 (|A||x|)_i error of a plain FP64 evaluation."""

import numpy as np
import pytest

import oracle as O
from sfem_gb300 import solvers as S
from sfem_gb300.mesh import SSMesh

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("with_low_part", [False, True])
@pytest.mark.parametrize("kind", ["laplacian", "elasticity"])
def test_compensated_residual_matches_oracle(cuda, kind, with_low_part):
    import torch

    vec = 3 if kind == "elasticity" else 1
    m = SSMesh(4, 3, 2, 4, perturb=0.1, seed=5)
    H = S.Hierarchy(m, dirichlet_faces=("x0",), device=cuda, vec=vec)
    res = S.CompensatedResidual(H, kind, mu=1.0, lam=10.0)
    em = res.em.cpu().numpy()
    el = m.elements(4)
    n = vec * m.n_nodes()
    rng = np.random.default_rng(6)
    x = rng.standard_normal(n)
    x_lo = 1e-17 * rng.standard_normal(n) if with_low_part else None
    dn = H.dirichlet[0].long().cpu().numpy()
    rows = (vec * dn[:, None] + np.arange(vec)[None, :]).reshape(-1)
    # b within 1e-9 of A x: the residual cancels almost completely
    b = -O.residual_dd_em(vec, 4, el, em, x, np.zeros(n)) + 1e-9 * rng.standard_normal(n)
    ref = O.residual_dd_em(vec, 4, el, em, x, b, x_lo=x_lo)
    ref[rows] = b[rows] - x[rows] - (x_lo[rows] if with_low_part else 0)
    xl = torch.from_numpy(x_lo).to(cuda) if with_low_part else None
    got = res(torch.from_numpy(x).to(cuda), torch.from_numpy(b).to(cuda), x_lo=xl).cpu().numpy()
    # residual entries ~1e-9, (|A||x|)_i = O(1): agreement to 4 ulp of the residual
    assert np.abs(got - ref).max() <= 4 * np.spacing(np.abs(ref).max()) + 1e-30
    # a plain FP64 evaluation misses by ~1e-16 of |A||x|, 1e7 times more
    if not with_low_part:
        plain = b - (-O.residual_dd_em(vec, 4, el, em, x, np.zeros(n)))
        assert np.abs(plain - ref)[~np.isin(np.arange(n), rows)].max() > 0


def test_dd_axpy_is_error_free(cuda):
    import torch

    rng = np.random.default_rng(7)
    hi = torch.from_numpy(rng.standard_normal(1000)).to(cuda)
    lo = torch.zeros_like(hi)
    e = torch.from_numpy(1e-12 * rng.standard_normal(1000)).to(cuda)
    h0 = hi.clone()
    S.dd_axpy(1.0, e, hi, lo)
    # (hi + lo) - h0 reproduces e exactly in exact arithmetic: check with the error terms
    d = ((hi - h0) + lo - e).abs().max().item()
    assert d == 0.0
