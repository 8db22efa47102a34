"""GPU parity of the matrix-free linear-elasticity operator against the CPU oracle."""

import numpy as np
import pytest

import oracle as O
from sfem_gb300 import capi
from sfem_gb300.mesh import SSMesh
from sfem_gb300.operators import SSMeshDevice

pytestmark = pytest.mark.gpu
MU, LAM = 1.0, 10.0


def _setup(cuda, L, n=(3, 2, 2), seed=0):
    import torch

    m = SSMesh(*n, L, box=((0, 4), (0, 1), (0, 1)), perturb=0.1, seed=seed)
    sp = SSMeshDevice(m, L, device=cuda)
    el = m.hex8_elements() if L == 1 else m.elements(L)
    corners = el if L == 1 else el[m.macro_corner_lidx(L)]
    adj, det = O.adjugate_fill(corners, m.points)
    adj_d = torch.from_numpy(adj.T.copy()).to(cuda)
    det_d = torch.from_numpy(det.copy()).to(cuda)
    return m, sp, el, adj, det, adj_d, det_d


def _scale(L, el, adj, det, u):
    # row scale (|K| |u|) bounded via the oracle on |u| plus the block-diagonal magnitude
    a = np.abs(O.linear_elasticity_apply(L if L > 1 else 0, el, adj, det, MU, LAM, np.abs(u)))
    d3, _ = O.linear_elasticity_block_diag(L if L > 1 else 0, el, adj, det, MU, LAM, u.size // 3)
    return a + 4 * np.abs(d3) * np.abs(u)


@pytest.mark.parametrize("L", [1, 2, 3, 4, 5, 8])
def test_elasticity_apply_fp64(cuda, L):
    import torch

    m, sp, el, adj, det, adj_d, det_d = _setup(cuda, L)
    n = m.n_nodes(L)
    rng = np.random.default_rng(L)
    u = rng.standard_normal(3 * n)
    y0 = rng.standard_normal(3 * n)
    ref = O.linear_elasticity_apply(L if L > 1 else 0, el, adj, det, MU, LAM, u, out=y0.copy())
    yd = torch.from_numpy(y0).to(cuda)
    ud = torch.from_numpy(u).to(cuda)
    capi.check(capi.load().sfem_gb300_linear_elasticity_apply(sp.element_type, capi.i64(m.n_elements),
                                                              sp.elements_ptrs.ptr, capi.i64(m.n_elements),
                                                              capi.vp(adj_d), capi.vp(det_d), ctypes_d(MU),
                                                              ctypes_d(LAM), capi.FLOAT64,
                                                              capi.vp(ud), capi.vp(yd), None),
               "elasticity apply")
    err = np.abs(yd.cpu().numpy() - ref) / (_scale(L, el, adj, det, u) + np.abs(y0))
    assert err.max() < 1e-13, err.max()


@pytest.mark.parametrize("L", [1, 2, 3])
def test_elasticity_apply_fp32_coarse_levels(cuda, L):
    """The float apply of the hex8 and L = 2, 3 levels (SIMT kernel) against the oracle."""
    import torch

    m, sp, el, adj, det, adj_d, det_d = _setup(cuda, L)
    n = m.n_nodes(L)
    rng = np.random.default_rng(10 + L)
    u = rng.standard_normal(3 * n)
    ref = O.linear_elasticity_apply(L if L > 1 else 0, el, adj, det, MU, LAM, u)
    yd = torch.zeros(3 * n, dtype=torch.float32, device=cuda)
    ud = torch.from_numpy(u).float().to(cuda)
    capi.check(capi.load().sfem_gb300_linear_elasticity_apply(sp.element_type, capi.i64(m.n_elements),
                                                              sp.elements_ptrs.ptr, capi.i64(m.n_elements),
                                                              capi.vp(adj_d), capi.vp(det_d), ctypes_d(MU),
                                                              ctypes_d(LAM), capi.FLOAT32,
                                                              capi.vp(ud), capi.vp(yd), None),
               "elasticity apply")
    err = np.abs(yd.double().cpu().numpy() - ref) / _scale(L, el, adj, det, u)
    assert err.max() < 2e-5, err.max()


@pytest.mark.parametrize("L,n", [(6, (2, 1, 1)), (16, (1, 1, 1))])
def test_elasticity_apply_fp32_high_levels(cuda, L, n):
    """Levels without a compile-time kernel (CTA per macro element) in FP32; FP64 at
    L = 16 needs more shared memory than a CTA has and is refused with a message."""
    import torch

    m, sp, el, adj, det, adj_d, det_d = _setup(cuda, L, n=n)
    nn = m.n_nodes(L)
    u = np.random.default_rng(30 + L).standard_normal(3 * nn)
    ref = O.linear_elasticity_apply(L, el, adj, det, MU, LAM, u)
    yd = torch.zeros(3 * nn, dtype=torch.float32, device=cuda)
    ud = torch.from_numpy(u).float().to(cuda)
    lib = capi.load()
    args = (sp.element_type, capi.i64(m.n_elements), sp.elements_ptrs.ptr, capi.i64(m.n_elements), capi.vp(adj_d),
            capi.vp(det_d), ctypes_d(MU), ctypes_d(LAM))
    capi.check(lib.sfem_gb300_linear_elasticity_apply(*args, capi.FLOAT32, capi.vp(ud), capi.vp(yd), None), "apply")
    err = np.abs(yd.double().cpu().numpy() - ref) / _scale(L, el, adj, det, u)
    assert err.max() < 2e-5, err.max()
    if L == 16:
        y64 = torch.zeros(3 * nn, dtype=torch.float64, device=cuda)
        u64 = torch.from_numpy(u).to(cuda)
        assert lib.sfem_gb300_linear_elasticity_apply(*args, capi.FLOAT64, capi.vp(u64), capi.vp(y64), None) == 1
        assert "shared memory" in capi.last_error()


@pytest.mark.parametrize("dtype_name,tol", [("float64", 1e-13), ("float32", 2e-5)])
@pytest.mark.parametrize("L", [1, 2, 3, 4])
def test_elasticity_stored_element_matrices(cuda, L, dtype_name, tol):
    """Element matrices stored once (coarse-level path) then applied: same operator as the
    oracle's, FP64 to 1e-13 and FP32 to 2e-5 of the row scale."""
    import torch

    m, sp, el, adj, det, adj_d, det_d = _setup(cuda, L, seed=5)
    n = m.n_nodes(L)
    dt = getattr(torch, dtype_name)
    rt = capi.FLOAT64 if dtype_name == "float64" else capi.FLOAT32
    rng = np.random.default_rng(20 + L)
    u = rng.standard_normal(3 * n)
    y0 = rng.standard_normal(3 * n)
    ref = O.linear_elasticity_apply(L if L > 1 else 0, el, adj, det, MU, LAM, u, out=y0.copy())
    lib = capi.load()
    E = m.n_elements
    K = torch.empty(576 * E, dtype=dt, device=cuda)
    capi.check(lib.sfem_gb300_linear_elasticity_element_matrices(sp.element_type, capi.i64(E), capi.i64(E),
                                                                  capi.vp(adj_d), capi.vp(det_d), ctypes_d(MU),
                                                                  ctypes_d(LAM), rt, capi.vp(K), None), "matrices")
    yd = torch.from_numpy(y0).to(dt).to(cuda)
    ud = torch.from_numpy(u).to(dt).to(cuda)
    capi.check(lib.sfem_gb300_linear_elasticity_apply_em(sp.element_type, capi.i64(E), sp.elements_ptrs.ptr,
                                                         capi.vp(K), rt, capi.vp(ud), capi.vp(yd), None), "apply_em")
    err = np.abs(yd.double().cpu().numpy() - ref) / (_scale(L, el, adj, det, u) + np.abs(y0))
    assert err.max() < tol, err.max()
    # the stored matrices are symmetric (built from the six distinct blocks)
    Kh = K.double().cpu().numpy().reshape(E, 24, 24)
    assert np.abs(Kh - Kh.transpose(0, 2, 1)).max() <= 1e-6 * np.abs(Kh).max()


def ctypes_d(v):
    import ctypes

    return ctypes.c_double(v)


@pytest.mark.parametrize("shape", [(3, 2, 2), (3, 3, 1)], ids=["12elements", "9elements"])
@pytest.mark.parametrize("fp32_kernel", [0, 1], ids=["simt", "tcgen05_3xtf32"])
def test_elasticity_reference_signature_and_fp32(cuda, fp32_kernel, shape):
    """FP64 = oracle to 1e-13; FP32 through the SIMT kernel or the tcgen05 3xTF32
    contraction (K and u split into TF32 hi + lo, hi.hi + hi.lo + lo.hi: FP32-level error)."""
    import torch

    L = 4
    m, sp, el, adj, det, adj_d, det_d = _setup(cuda, L, n=shape, seed=3)
    n = m.n_nodes(L)
    u = np.random.default_rng(5).standard_normal(3 * n)
    ref = O.linear_elasticity_apply(L, el, adj, det, MU, LAM, u)
    lib = capi.load()
    capi.check(lib.sfem_gb300_set_elasticity_kernel(fp32_kernel), "variant")
    # FLOAT32: FP32 SIMT contraction.  FLOAT32_BF16TC: tensor-core BF16 contraction with FP32
    # accumulate; K and u rounded to 8-bit mantissas (2^-8 per product) against a row scale that
    # underestimates sum |K_ij||u_j| several-fold: 2.8e-2 observed, bounded here by 6e-2.
    for dt, rt, tol in ((torch.float64, capi.FLOAT64, 1e-13), (torch.float32, capi.FLOAT32, 2e-5),
                        (torch.float32, capi.FLOAT32_BF16TC, 6e-2)):
        ud = torch.from_numpy(u).to(cuda).to(dt)
        yd = torch.zeros(3 * n, dtype=dt, device=cuda)
        es = ud.element_size()
        capi.check(lib.cu_affine_sshex8_linear_elasticity_apply(
            L, capi.i64(m.n_elements), sp.elements_ptrs.ptr, capi.i64(m.n_elements), capi.vp(adj_d), capi.vp(det_d),
            ctypes_d(MU), ctypes_d(LAM), rt, capi.i64(3), capi.vp(ud), capi.c_void(ud.data_ptr() + es),
            capi.c_void(ud.data_ptr() + 2 * es), capi.i64(3), capi.vp(yd), capi.c_void(yd.data_ptr() + es),
            capi.c_void(yd.data_ptr() + 2 * es), None), "cu_affine_sshex8_linear_elasticity_apply")
        err = np.abs(yd.double().cpu().numpy() - ref) / _scale(L, el, adj, det, u)
        assert err.max() < tol, (dt, rt, err.max())
    capi.check(lib.sfem_gb300_set_elasticity_kernel(-1), "variant")
    assert lib.sfem_gb300_elasticity_status() == 0
    # other layouts, as the reference's signature allows: separate component arrays
    # (stride 1) and interleaved with a padding slot (stride 4); the padding stays untouched
    for dt, rt, tol in ((torch.float64, capi.FLOAT64, 1e-13), (torch.float32, capi.FLOAT32, 2e-5)):
        for stride in (1, 4):
            if stride == 1:
                us = [torch.from_numpy(u[d::3].copy()).to(cuda).to(dt) for d in range(3)]
                ys = [torch.zeros(n, dtype=dt, device=cuda) for _ in range(3)]
                uptr, yptr = [capi.vp(t) for t in us], [capi.vp(t) for t in ys]
            else:
                ub = torch.full((n, 4), 7.0, dtype=dt, device=cuda)
                ub[:, :3] = torch.from_numpy(u.reshape(n, 3)).to(cuda).to(dt)
                yb = torch.full((n, 4), -3.0, dtype=dt, device=cuda)
                yb[:, :3] = 0
                es = ub.element_size()
                uptr = [capi.c_void(ub.data_ptr() + d * es) for d in range(3)]
                yptr = [capi.c_void(yb.data_ptr() + d * es) for d in range(3)]
            capi.check(lib.cu_affine_sshex8_linear_elasticity_apply(
                L, capi.i64(m.n_elements), sp.elements_ptrs.ptr, capi.i64(m.n_elements), capi.vp(adj_d),
                capi.vp(det_d), ctypes_d(MU), ctypes_d(LAM), rt, capi.i64(stride), *uptr, capi.i64(stride), *yptr,
                None), "cu_affine_sshex8_linear_elasticity_apply (strided)")
            torch.cuda.synchronize()
            if stride == 1:
                got = torch.stack(ys, dim=1).reshape(-1)
            else:
                assert bool((yb[:, 3] == -3.0).all())
                got = yb[:, :3].reshape(-1)
            err = np.abs(got.double().cpu().numpy() - ref) / _scale(L, el, adj, det, u)
            assert err.max() < tol, (dt, stride, err.max())


@pytest.mark.parametrize("L", [1, 2, 4, 8])
def test_elasticity_block_diag(cuda, L):
    import torch

    m, sp, el, adj, det, adj_d, det_d = _setup(cuda, L, seed=7)
    n = m.n_nodes(L)
    d3_ref, b6_ref = O.linear_elasticity_block_diag(L if L > 1 else 0, el, adj, det, MU, LAM, n)
    d3 = torch.zeros(3 * n, dtype=torch.float64, device=cuda)
    b6 = torch.zeros(6 * n, dtype=torch.float64, device=cuda)
    capi.check(capi.load().sfem_gb300_linear_elasticity_block_diag(
        sp.element_type, capi.i64(m.n_elements), sp.elements_ptrs.ptr, capi.i64(m.n_elements), capi.vp(adj_d),
        capi.vp(det_d), ctypes_d(MU), ctypes_d(LAM), capi.FLOAT64, capi.vp(d3), capi.vp(b6), None), "block diag")
    assert np.abs(d3.cpu().numpy() - d3_ref).max() <= 1e-13 * np.abs(d3_ref).max()
    assert np.abs(b6.cpu().numpy() - b6_ref).max() <= 1e-13 * np.abs(b6_ref).max()
