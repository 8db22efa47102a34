"""Host-side mesh hierarchy logic: macro-grid coarse hex8 levels and their transfer arrays,
checked with the oracle's restatement of the sshex8 transfer."""

import numpy as np

import oracle as O
from sfem_gb300.mesh import SSMesh, macro_coarse_levels, macro_level_grid


def test_macro_coarse_levels_shapes():
    m = SSMesh(48, 48, 48, 4)
    assert [l.shape for l in macro_coarse_levels(m)] == [(24, 24, 24), (12, 12, 12), (6, 6, 6), (3, 3, 3)]
    m = SSMesh(64, 16, 16, 4)
    assert [l.shape for l in macro_coarse_levels(m)] == [(32, 8, 8), (16, 4, 4), (8, 2, 2)]
    assert macro_coarse_levels(SSMesh(5, 4, 4, 2)) == []


def test_macro_coarse_transfer_is_trilinear_and_adjoint():
    m = SSMesh(8, 4, 8, 2, perturb=0.1, seed=3)
    pts, ids = macro_level_grid(m)
    levels = macro_coarse_levels(m, min_nodes=8)
    assert len(levels) == 2
    fine_ids = ids
    n_fine = m.n_nodes(1)
    rng = np.random.default_rng(0)
    for lvl in levels:
        # coarse geometry = finer grid nodes at even positions
        cz, cy, cx = lvl.ids.shape
        np.testing.assert_array_equal(lvl.points_grid, pts[:, ::2, ::2, ::2])
        # linear functions in index space are interpolated exactly
        K, J, I = np.meshgrid(np.arange(cz), np.arange(cy), np.arange(cx), indexing="ij")
        xc = (1 + 2 * I - J + 0.5 * K).reshape(-1).astype(np.float64)
        yf = O.prolongate(1, lvl.from_lidx, 2, lvl.to_lidx, 1, xc, n_fine)
        fz, fy, fx = fine_ids.shape
        K, J, I = np.meshgrid(np.arange(fz), np.arange(fy), np.arange(fx), indexing="ij")
        want = np.zeros(n_fine)
        want[fine_ids.reshape(-1)] = (1 + I - J / 2 + K / 4).reshape(-1)
        np.testing.assert_allclose(yf, want, rtol=0, atol=1e-12)
        # restriction is the transpose of prolongation (vector of 3 too)
        for vec in (1, 3):
            xf = rng.standard_normal(vec * n_fine)
            xc = rng.standard_normal(vec * lvl.n_nodes)
            Px = O.prolongate(1, lvl.from_lidx, 2, lvl.to_lidx, vec, xc, n_fine)
            Rx = O.restrict(2, lvl.to_lidx, lvl.fine_count, 1, lvl.from_lidx, vec, xf, lvl.n_nodes)
            assert abs(xf @ Px - Rx @ xc) <= 1e-12 * abs(xf @ Px)
        # boundary faces
        assert lvl.boundary_nodes("x0").size == (cy * cz)
        fine_ids, pts, n_fine = lvl.ids, lvl.points_grid, lvl.n_nodes


def test_draw_problems_is_seeded_and_in_range():
    from sfem_gb300.batch import draw_problems

    a = draw_problems(256, seed=3)
    assert a == draw_problems(256, seed=3) and a != draw_problems(256, seed=4)
    assert all(8 <= p.n <= 32 and p.level in (2, 3, 4) for p in a)
    kinds = {p.kind for p in a}
    assert kinds == {"poisson", "elasticity"}
    assert len({p.seed for p in a}) == 256
