"""Symmetric CRS / BSR SpMV and the hex8 Laplacian CRS assembly against the oracle."""

import ctypes

import numpy as np
import pytest

import oracle as O
from sfem_gb300 import capi
from sfem_gb300.mesh import SSMesh, upper_crs_graph
from sfem_gb300.operators import SSMeshDevice

pytestmark = pytest.mark.gpu
D = ctypes.c_double


def _t(a, cuda):
    import torch

    return torch.from_numpy(np.ascontiguousarray(a)).to(cuda)


def test_hex8_laplacian_crs_sym_assembly_and_spmv(cuda):
    import torch

    m = SSMesh(6, 5, 4, 1, perturb=0.2, seed=3)
    el = m.hex8_elements()
    n = m.n_nodes(1)
    rowptr, colidx = upper_crs_graph(el, n)
    fff = O.fff_fill(el, m.points)
    d_ref, o_ref = O.hex8_laplacian_crs_sym(el, fff, rowptr, colidx, n)
    if O.ref() is not None:  # the oracle assembly is pinned to the reference's
        d_r, o_r = O.hex8_laplacian_crs_sym(el, fff, rowptr, colidx, n, use_ref=True, points=m.points)
        assert np.abs(d_r - d_ref).max() <= 1e-6 * np.abs(d_r).max()  # reference uses unrounded geometry
    sp = SSMeshDevice(m, 1, device=cuda)
    fff_d = _t(fff.T, cuda)
    rp, ci = _t(rowptr, cuda), _t(colidx, cuda)
    diag = torch.zeros(n, dtype=torch.float64, device=cuda)
    off = torch.zeros(colidx.size, dtype=torch.float64, device=cuda)
    lib = capi.load()
    capi.check(lib.sfem_gb300_hex8_laplacian_crs_sym(capi.i64(m.n_elements), sp.elements_ptrs.ptr,
                                                     capi.i64(m.n_elements), capi.vp(fff_d), capi.vp(rp), capi.vp(ci),
                                                     capi.FLOAT64, capi.vp(diag), capi.vp(off), None), "assembly")
    assert np.abs(diag.cpu().numpy() - d_ref).max() <= 1e-13 * np.abs(d_ref).max()
    assert np.abs(off.cpu().numpy() - o_ref).max() <= 1e-13 * np.abs(o_ref).max()
    # SpMV == matrix-free apply
    x = np.random.default_rng(0).standard_normal(n)
    y_mf = O.hex8_laplacian_apply(el, fff, x)
    y_or = O.crs_sym_spmv(rowptr, colidx, d_ref, o_ref, x)
    assert np.abs(y_or - y_mf).max() <= 1e-12 * np.abs(y_mf).max()
    y = torch.full((n,), 3.0, dtype=torch.float64, device=cuda)
    x_d = _t(x, cuda)
    capi.check(lib.sfem_gb300_crs_sym_spmv(capi.FLOAT64, capi.i64(n), capi.vp(rp), capi.vp(ci), capi.vp(diag),
                                           capi.vp(off), D(0.5), capi.vp(x_d), capi.vp(y), None), "spmv")
    assert np.abs(y.cpu().numpy() - (1.5 + y_or)).max() <= 1e-12 * np.abs(y_or).max()


@pytest.mark.parametrize("bs,sym", [(3, 0), (3, 1), (2, 0)])
def test_bsr_sym_spmv(cuda, bs, sym):
    import torch

    rng = np.random.default_rng(bs + 10 * sym)
    nb = 500
    # random upper block graph
    rows, cols = [], []
    for i in range(nb):
        c = np.unique(rng.integers(i + 1, nb, size=5)) if i + 1 < nb else np.array([], int)
        rows += [i] * len(c)
        cols += list(c)
    rowptr = np.zeros(nb + 1, dtype=np.int32)
    np.add.at(rowptr, np.array(rows, dtype=np.int64) + 1, 1)
    rowptr = np.cumsum(rowptr).astype(np.int32)
    colidx = np.array(cols, dtype=np.int32)
    ns = bs * (bs + 1) // 2
    dsym = rng.standard_normal(nb * ns)
    nnz = colidx.size
    if sym:
        off_s = rng.standard_normal(nnz * ns)
        off_full = np.zeros((nnz, bs, bs))
        k = 0
        for a in range(bs):
            for b in range(a, bs):
                off_full[:, a, b] = off_s[k::ns]
                off_full[:, b, a] = off_s[k::ns]
                k += 1
        off_in = off_s
        off_full = off_full.reshape(-1)
    else:
        off_full = rng.standard_normal(nnz * bs * bs)
        off_in = off_full
    x = rng.standard_normal(nb * bs)
    ref = O.bsr_sym_spmv(bs, rowptr, colidx, dsym, off_full, x)
    y = torch.zeros(nb * bs, dtype=torch.float64, device=cuda)
    # keep every device array referenced until the kernel has run (no temporaries whose
    # memory the caching allocator could hand to the next argument)
    rp_d, ci_d, d_d, o_d, x_d = (_t(a, cuda) for a in (rowptr, colidx, dsym, off_in, x))
    capi.check(capi.load().sfem_gb300_bsr_sym_spmv(capi.FLOAT64, bs, capi.i64(nb), capi.vp(rp_d), capi.vp(ci_d),
                                                   capi.vp(d_d), capi.vp(o_d), sym, D(0.0), capi.vp(x_d), capi.vp(y),
                                                   None), "bsr")
    torch.cuda.synchronize()
    assert np.abs(y.cpu().numpy() - ref).max() <= 1e-12 * np.abs(ref).max()


def _csr_matvec(rowptr, colidx, vals, x, bs=1):
    n = rowptr.size - 1
    y = np.zeros(n * bs)
    blocks = vals.reshape(-1, bs, bs)
    for i in range(n):
        for k in range(rowptr[i], rowptr[i + 1]):
            y[i * bs:(i + 1) * bs] += blocks[k] @ x[colidx[k] * bs:(colidx[k] + 1) * bs]
    return y


def test_reference_named_laplacian_assembly(cuda):
    """cu_laplacian_crs (full graph) and cu_laplacian_crs_sym under the reference's names:
    the assembled matrices reproduce the matrix-free oracle apply; other element types
    are refused with a message."""
    import torch

    from sfem_gb300.mesh import full_crs_graph

    m = SSMesh(5, 4, 3, 1, perturb=0.2, seed=4)
    el = m.hex8_elements()
    n = m.n_nodes(1)
    fff = O.fff_fill(el, m.points)
    sp = SSMeshDevice(m, 1, device=cuda)
    fff_d = _t(fff.T, cuda)
    E = m.n_elements
    lib = capi.load()
    x = np.random.default_rng(1).standard_normal(n)
    y_mf = O.hex8_laplacian_apply(el, fff, x)
    rowptr, colidx = full_crs_graph(el, n)
    rp, ci = _t(rowptr, cuda), _t(colidx, cuda)
    vals = torch.zeros(colidx.size, dtype=torch.float64, device=cuda)
    capi.check(lib.cu_laplacian_crs(capi.HEX8, capi.i64(E), sp.elements_ptrs.ptr, capi.i64(E), capi.vp(fff_d),
                                    capi.vp(rp), capi.vp(ci), capi.FLOAT64, capi.vp(vals), None), "cu_laplacian_crs")
    y = _csr_matvec(rowptr, colidx, vals.cpu().numpy(), x)
    assert np.abs(y - y_mf).max() <= 1e-12 * np.abs(y_mf).max()
    urp, uci = upper_crs_graph(el, n)
    urp_d, uci_d = _t(urp, cuda), _t(uci, cuda)
    diag = torch.zeros(n, dtype=torch.float64, device=cuda)
    off = torch.zeros(uci.size, dtype=torch.float64, device=cuda)
    capi.check(lib.cu_laplacian_crs_sym(capi.HEX8, capi.i64(E), sp.elements_ptrs.ptr, capi.i64(E), capi.vp(fff_d),
                                        capi.vp(urp_d), capi.vp(uci_d), capi.FLOAT64, capi.vp(diag), capi.vp(off),
                                        None), "cu_laplacian_crs_sym")
    y2 = O.crs_sym_spmv(urp, uci, diag.cpu().numpy(), off.cpu().numpy(), x)
    assert np.abs(y2 - y_mf).max() <= 1e-12 * np.abs(y_mf).max()
    assert lib.cu_laplacian_crs(capi.SSHEX8(2), capi.i64(E), sp.elements_ptrs.ptr, capi.i64(E), capi.vp(fff_d),
                                capi.vp(rp), capi.vp(ci), capi.FLOAT64, capi.vp(vals), None) == 1
    assert "HEX8" in capi.last_error()


def test_reference_named_elasticity_entry_points(cuda):
    """cu_linear_elasticity_apply / _diag / _block_diag_sym_aos / _bsr against the oracle
    (hex8 and sshex8 L = 2; BSR on hex8 as the reference)."""
    import torch

    from sfem_gb300.mesh import full_crs_graph

    mu, lam = 1.0, 10.0
    lib = capi.load()
    for L in (1, 2):
        m = SSMesh(4, 3, 2, L, box=((0, 4), (0, 1), (0, 1)), perturb=0.1, seed=L)
        sp = SSMeshDevice(m, L, device=cuda)
        el = m.hex8_elements() if L == 1 else m.elements(L)
        corners = el if L == 1 else el[m.macro_corner_lidx(L)]
        adj, det = O.adjugate_fill(corners, m.points)
        adj_d, det_d = _t(adj.T, cuda), _t(det, cuda)
        n = m.n_nodes(L)
        E = m.n_elements
        et = capi.HEX8 if L == 1 else capi.SSHEX8(L)
        Lo = 0 if L == 1 else L
        u = np.random.default_rng(2).standard_normal(3 * n)
        ref = O.linear_elasticity_apply(Lo, el, adj, det, mu, lam, u)
        y = torch.zeros(3 * n, dtype=torch.float64, device=cuda)
        capi.check(lib.cu_linear_elasticity_apply(et, capi.i64(E), sp.elements_ptrs.ptr, capi.i64(E), capi.vp(adj_d),
                                                  capi.vp(det_d), D(mu), D(lam), capi.FLOAT64, capi.vp(_t(u, cuda)),
                                                  capi.vp(y), None), "apply")
        scale = O.linear_elasticity_row_scale(Lo, el, adj, det, mu, lam, u)
        assert (np.abs(y.cpu().numpy() - ref) / scale).max() < 1e-13
        d3_ref, b6_ref = O.linear_elasticity_block_diag(Lo, el, adj, det, mu, lam, n)
        d3 = torch.zeros(3 * n, dtype=torch.float64, device=cuda)
        b6 = torch.zeros(6 * n, dtype=torch.float64, device=cuda)
        capi.check(lib.cu_linear_elasticity_diag(et, capi.i64(E), sp.elements_ptrs.ptr, capi.i64(E), capi.vp(adj_d),
                                                 capi.vp(det_d), D(mu), D(lam), capi.FLOAT64, capi.vp(d3), None), "diag")
        capi.check(lib.cu_linear_elasticity_block_diag_sym_aos(et, capi.i64(E), sp.elements_ptrs.ptr, capi.i64(E),
                                                               capi.vp(adj_d), capi.vp(det_d), D(mu), D(lam),
                                                               capi.FLOAT64, capi.vp(b6), None), "block diag")
        assert np.abs(d3.cpu().numpy() - d3_ref).max() <= 1e-13 * np.abs(d3_ref).max()
        assert np.abs(b6.cpu().numpy() - b6_ref).max() <= 1e-13 * np.abs(b6_ref).max()
        if L == 1:
            rowptr, colidx = full_crs_graph(el, n)
            rp, ci = _t(rowptr, cuda), _t(colidx, cuda)
            vals = torch.zeros(colidx.size * 9, dtype=torch.float64, device=cuda)
            capi.check(lib.cu_linear_elasticity_bsr(et, capi.i64(E), sp.elements_ptrs.ptr, capi.i64(E),
                                                    capi.vp(adj_d), capi.vp(det_d), D(mu), D(lam), capi.FLOAT64,
                                                    capi.vp(rp), capi.vp(ci), capi.vp(vals), None), "bsr")
            yb = _csr_matvec(rowptr, colidx, vals.cpu().numpy(), u, bs=3)
            assert (np.abs(yb - ref) / scale).max() < 1e-13
            # symmetric blocks: the (i, j) block is the transpose of (j, i)
            V = vals.cpu().numpy().reshape(-1, 3, 3)
            k = 5
            row = np.searchsorted(rowptr, k, side="right") - 1
            col = colidx[k]
            kt = rowptr[col] + np.searchsorted(colidx[rowptr[col]:rowptr[col + 1]], row)
            assert np.abs(V[k] - V[kt].T).max() <= 1e-15 * np.abs(V).max()
