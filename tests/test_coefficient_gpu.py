"""Variable coefficient k = exp(g) (per macro element, folded into the metric) on the GPU:
the apply equals the reference's stencil apply on FFF * k_e (committed fixture, produced
by the reference's own kernel), and a multigrid solve with k matches the CPU oracle's
solve of the same problem."""

from pathlib import Path

import numpy as np
import pytest

import oracle as O
from sfem_gb300.mesh import SSMesh
from sfem_gb300.operators import Laplacian, SSMeshDevice

pytestmark = pytest.mark.gpu
COEF = Path(__file__).resolve().parent / "golden" / "sshex8_coefficient.npz"


@pytest.mark.parametrize("dtype_name,tol", [("float64", 1e-13), ("float32", 2e-5)])
def test_coefficient_apply_matches_reference(cuda, dtype_name, tol):
    import torch

    g = np.load(COEF)
    m = SSMesh(int(g["nx"]), int(g["ny"]), int(g["nz"]), int(g["level"]), perturb=float(g["perturb"]),
               seed=int(g["seed"]))
    assert np.array_equal(m.elements(4), g["elements"])
    sp = SSMeshDevice(m, 4, device=cuda)
    op = Laplacian(sp, coefficient=g["k"]).initialize()
    # the operator's own metric: computed on the GPU from the coordinates, then scaled
    fffk = op.fff.cpu().numpy().T
    assert np.abs(fffk - g["fff_scaled"]).max() <= 2.5e-7 * np.abs(g["fff_scaled"]).max()
    dt = getattr(torch, dtype_name)
    x = torch.from_numpy(g["x"]).to(dt).to(cuda)
    y = torch.zeros_like(x)
    op.apply(x, y)
    ref = O.sshex8_laplacian_stencil_apply(4, g["elements"], fffk.copy(), g["x"])
    ax = np.abs(O.sshex8_laplacian_stencil_apply(4, g["elements"], fffk.copy(), np.abs(g["x"])))
    scale = ax + 2 * O.laplacian_diag(4, g["elements"], fffk.copy(), g["x"].size) * np.abs(g["x"])
    assert (np.abs(y.double().cpu().numpy() - ref) / scale).max() < tol
    # and the reference's own output (its FFF from the same coordinates, computed on the host)
    assert (np.abs(y.double().cpu().numpy() - g["laplacian_apply"]) / scale).max() < max(tol, 1e-6)


def test_coefficient_solve_matches_cpu_oracle(cuda):
    import torch

    from sfem_gb300 import solvers as S
    from sfem_gb300.coefficients import lognormal_coefficient

    m = SSMesh(8, 8, 8, 4, perturb=0.1, seed=44)
    k = lognormal_coefficient(8, 8, 8, ell=2.0, sigma=1.0, seed=45)
    H = S.Hierarchy(m, dirichlet_faces=("x0",), device=cuda, coefficient=k, coarsen_macro=True)
    b = np.random.default_rng(46).standard_normal(m.n_nodes())
    dn = H.dirichlet[0].long().cpu().numpy()
    b[dn] = 0
    ctx = S.context()
    op64 = S.laplacian_op(ctx, H.spaces[0], H.fff, H.dirichlet[0], torch.float64)
    mg, _ = S.build_poisson_mg(ctx, H, torch.float64, smoother="chebyshev3", sweeps=2, coarse="dense")
    cg = S.cg(ctx, op64, mg, rtol=1e-11, max_it=200, residual_norm=True, flexible=True)
    bd = torch.from_numpy(b).to(cuda)
    x = torch.zeros_like(bd)
    assert S.solve(cg, bd, x) == 0
    fffk = H.fff.cpu().numpy().T.copy()
    xc, st = O.mg_pcg_solve(m, "laplacian", b, geom=fffk, rtol=1e-11, flexible=True)
    assert st["rc"] == 0
    xg = x.cpu().numpy()
    assert np.linalg.norm(xg - xc) <= 1e-8 * np.linalg.norm(xc)
    res = S.CompensatedResidual(H, "laplacian")
    assert res.relative(x, bd) <= 1.5e-11
