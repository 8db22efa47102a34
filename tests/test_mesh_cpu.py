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
    # odd edges keep a thin last element
    assert [l.shape for l in macro_coarse_levels(SSMesh(31, 31, 31, 1))] == [(16, 16, 16), (8, 8, 8), (4, 4, 4)]
    assert macro_coarse_levels(SSMesh(5, 4, 4, 2)) == []


def _csr_dense(csr, nrows, ncols):
    rp, ci, w = csr
    M = np.zeros((nrows, ncols))
    for i in range(nrows):
        M[i, ci[rp[i]:rp[i + 1]]] += w[rp[i]:rp[i + 1]]
    return M


def test_macro_coarse_transfer_is_trilinear_and_adjoint():
    for dims in ((8, 4, 8), (7, 5, 6)):
        m = SSMesh(*dims, 2, perturb=0.1, seed=3)
        pts, ids = macro_level_grid(m)
        levels = macro_coarse_levels(m, min_nodes=8)
        assert len(levels) >= 1
        fine_ids, n_fine = ids, m.n_nodes(1)
        fpts = pts
        for lvl in levels:
            P = _csr_dense(lvl.P, n_fine, lvl.n_nodes)
            R = _csr_dense(lvl.R, lvl.n_nodes, n_fine)
            np.testing.assert_array_equal(R, P.T)
            np.testing.assert_allclose(P.sum(axis=1), 1.0, rtol=0, atol=1e-14)  # partition of unity
            # coarse nodes are finer nodes (nested): their coordinates are copied exactly
            fz, fy, fx = fine_ids.shape
            flat_pts = np.empty((3, n_fine), dtype=np.float32)
            flat_pts[:, fine_ids.reshape(-1)] = fpts.reshape(3, -1)
            np.testing.assert_array_equal((P.T @ np.ones(n_fine) > 0).sum(), lvl.n_nodes)
            # linear functions of the finer grid's physical coordinates are reproduced on the
            # finer nodes by interpolating their coarse-node values (affine along each axis)
            for d in range(3):
                coarse_vals = lvl.points[d].astype(np.float64)
                # index-space linear function: exact for any (non-uniform) nesting
                K, J, I = np.meshgrid(np.arange(fz), np.arange(fy), np.arange(fx), indexing="ij")
                f_fine = np.zeros(n_fine)
                f_fine[fine_ids.reshape(-1)] = (1 + 2 * I - J + 0.5 * K).reshape(-1)
                kept = [np.asarray(sorted(set(range(0, n + 1, 2)) | {n})) for n in (fx - 1, fy - 1, fz - 1)]
                CZ, CY, CX = np.meshgrid(kept[2], kept[1], kept[0], indexing="ij")
                f_coarse = (1 + 2 * CX - CY + 0.5 * CZ).reshape(-1)
                np.testing.assert_allclose(P @ f_coarse, f_fine, rtol=0, atol=1e-12)
            assert lvl.boundary_nodes("x0").size == (lvl.shape[1] + 1) * (lvl.shape[2] + 1)
            fine_ids, n_fine, fpts = lvl.ids, lvl.n_nodes, lvl.points_grid


def test_draw_problems_is_seeded_and_in_range():
    from sfem_gb300.batch import draw_problems

    a = draw_problems(256, seed=3)
    assert a == draw_problems(256, seed=3) and a != draw_problems(256, seed=4)
    assert all(8 <= p.n <= 32 and p.level in (2, 3, 4) for p in a)
    kinds = {p.kind for p in a}
    assert kinds == {"poisson", "elasticity"}
    assert len({p.seed for p in a}) == 256
