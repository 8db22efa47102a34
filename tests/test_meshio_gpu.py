"""Meshes read from reference mesh folders through the GPU path: the fixture written
by the reference's own box_mesh.py, and a perturbed macro mesh with scrambled node
numbering and rotated element corner orders written and read back.  Operator
parity against the oracle and multigrid solves to the true FP64 residual 1e-10."""

from pathlib import Path

import numpy as np
import pytest

import oracle as O
import oracle.solvers as OS
from sfem_gb300 import solvers as S
from sfem_gb300.mesh import HEX8_CORNERS, SSMesh
from sfem_gb300.meshio import SfemMesh, ssmesh_from_folder, write_sfem_mesh
from sfem_gb300.operators import Laplacian

pytestmark = pytest.mark.gpu

FIXTURE = Path(__file__).resolve().parent / "golden" / "box_mesh_hex8"


def _scrambled_folder(path, n=(6, 5, 4), perturb=0.2, seed=3):
    """A perturbed n[0] x n[1] x n[2] macro mesh with random node ids and element
    corner orders (random rotations of the reference cube), written as a mesh folder
    with the boundary node set 'left' (x = 0)."""
    m = SSMesh(*n, 1, perturb=perturb, seed=seed)
    el = m.hex8_elements()
    pts = m.points
    rng = np.random.default_rng(seed)
    newid = rng.permutation(pts.shape[1])
    p2 = np.empty_like(pts)
    p2[:, newid] = pts
    el = newid[el]
    rots = []
    for perm in ([0, 1, 2], [0, 2, 1], [1, 0, 2], [1, 2, 0], [2, 0, 1], [2, 1, 0]):
        for signs in np.ndindex(2, 2, 2):
            R = np.zeros((3, 3), dtype=int)
            for i in range(3):
                R[i, perm[i]] = 1 - 2 * signs[i]
            if round(np.linalg.det(R)) == 1:
                rots.append(R)
    key = {tuple(c): k for k, c in enumerate(HEX8_CORNERS)}
    out = np.empty_like(el)
    for e in range(el.shape[1]):
        R = rots[rng.integers(len(rots))]
        for k in range(8):
            out[k, e] = el[key[tuple((R @ (2 * HEX8_CORNERS[k] - 1) + 1) // 2)], e]
    left = newid[np.flatnonzero(np.isclose(pts[0], 0.0))]
    write_sfem_mesh(path, SfemMesh("HEX8", out, p2, {"left": left}))


def _oracle(hm, L, fff, dn):
    el = hm.elements(L)

    def apply(x):
        y = O.sshex8_laplacian_apply(L, el, fff, x)
        y[dn] = x[dn]
        return y

    d = O.laplacian_diag(L, el, fff, hm.n_nodes(L))
    d[dn] = 1
    return apply, d


@pytest.mark.parametrize("source", ["reference_box", "scrambled"])
def test_mesh_folder_poisson(cuda, tmp_path, source):
    import torch

    L = 4
    folder = FIXTURE
    if source == "scrambled":
        folder = tmp_path / "mesh"
        _scrambled_folder(folder)
    hm = ssmesh_from_folder(folder, L)
    H = S.Hierarchy(hm, dirichlet_faces=("left",), device=cuda)
    fff = H.fff.cpu().numpy().T.copy()
    dn = H.dirichlet[0].cpu().numpy()
    assert dn.size > 0
    apply, d = _oracle(hm, L, fff, dn)
    # operator parity, FP64 (1e-13 of the row scale) and FP32 (packed tiles, 2e-5)
    el = hm.elements(L)
    x = np.random.default_rng(1).standard_normal(hm.n_nodes(L))
    ref = O.sshex8_laplacian_apply(L, el, fff, x)
    scale = np.abs(O.sshex8_laplacian_apply(L, el, fff, np.abs(x))) + 2 * O.laplacian_diag(L, el, fff, x.size) * np.abs(x)
    op = Laplacian(H.spaces[0]).set_fff(H.fff)
    assert op.packed_blocks is not None
    for dt, tol in ((torch.float64, 1e-13), (torch.float32, 2e-5)):
        y = torch.zeros(x.size, dtype=dt, device=cuda)
        op.apply(torch.from_numpy(x).to(dt).to(cuda), y)
        assert (np.abs(y.double().cpu().numpy() - ref) / scale).max() < tol, dt
    # FP64 MG-PCG and FP64 flexible CG over the FP32 multigrid, both to 1e-10
    b = np.random.default_rng(2).standard_normal(hm.n_nodes(L))
    b[dn] = 0
    x_star, _ = OS.cg(apply, b, precond=lambda r: r / d, rtol=1e-14, max_it=20000)
    bd = torch.from_numpy(b).to(cuda)
    ctx = S.context()
    mg, op64 = S.build_poisson_mg(ctx, H, torch.float64, sweeps=2)
    solver = S.cg(ctx, op64, mg, rtol=1e-11, max_it=100, residual_norm=True)
    xd = torch.zeros_like(bd)
    assert S.solve(solver, bd, xd) == 0
    mg32, _ = S.build_poisson_mg(ctx, H, torch.float32, sweeps=2)
    fcg = S.cg(ctx, op64, S.mixed_precond(ctx, mg32), rtol=1e-11, max_it=100, residual_norm=True, flexible=True)
    xm = torch.zeros_like(bd)
    assert S.solve(fcg, bd, xm) == 0
    for sol in (xd, xm):
        xs = sol.cpu().numpy()
        assert np.linalg.norm(b - apply(xs)) / np.linalg.norm(b) <= 1.01e-10
        assert np.linalg.norm(xs - x_star) <= 1e-6 * np.linalg.norm(x_star)
