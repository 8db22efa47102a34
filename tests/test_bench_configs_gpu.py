"""Parity at the benchmark sizes.

* Poisson mesh: 48^3 macro hex8 elements of the unit cube at L = 4 (110,592 macro
  elements, 7,189,057 nodes), interior macro nodes perturbed by U(-0.1, 0.1) h, seed 0
  -- the mesh of the benchmark's apply step and of its Poisson solves.
* Cantilever: 64 x 16 x 16 macro elements of [0,4] x [0,1] x [0,1] at L = 4 (16,384 macro
  elements, 3,257,475 dofs), mu = 1, lambda = 10.

Every GPU form of the operator is compared with the CPU oracle (the stencil-form
restatement of affine_sshex8_laplacian_stencil_apply_fff and the restatement of
affine_sshex8_linear_elasticity_apply_macro_adjugate, both pinned to the reference's
own kernels).  Tolerances, per entry against the row scale (|A| |x|)_i: FP64 1e-13;
FP32 2e-5 (float rounding of the metric, the coefficients and the sums).
"""

import numpy as np
import pytest

import oracle as O
from sfem_gb300 import capi
from sfem_gb300.mesh import SSMesh
from sfem_gb300.operators import Laplacian, SSMeshDevice

pytestmark = pytest.mark.gpu

RTOL64 = 1e-13
RTOL32 = 2e-5
MU, LAM = 1.0, 10.0


@pytest.fixture(scope="module")
def cube48(cuda):
    import torch

    L = 4
    m = SSMesh(48, 48, 48, L, perturb=0.1, seed=0)
    el = m.elements(L)
    fff = O.fff_fill(el[m.macro_corner_lidx(L)], m.points)
    sp = SSMeshDevice(m, L, device=cuda)
    op = Laplacian(sp, packed=True).set_fff(torch.from_numpy(fff.T.copy()))
    x = np.random.default_rng(1).standard_normal(m.n_nodes())
    ref = O.sshex8_laplacian_stencil_apply(L, el, fff, x)
    scale = np.abs(O.sshex8_laplacian_stencil_apply(L, el, fff, np.abs(x)))
    scale += 2 * O.laplacian_diag(L, el, fff, m.n_nodes()) * np.abs(x)
    return dict(m=m, el=el, fff=fff, sp=sp, op=op, x=x, ref=ref, scale=scale)


@pytest.mark.parametrize("form", ["soa_default", "packed", "warp_element_matrix"])
def test_cube48_fp64_apply(cuda, cube48, form):
    """FP64 on the 48^3 L = 4 mesh: the stencil kernel from SoA rows (cu_laplacian_apply
    default) and from packed tiles (the operator), and the warp element-matrix kernel."""
    import torch

    c = cube48
    lib = capi.load()
    x = torch.from_numpy(c["x"]).to(cuda)
    y = torch.zeros_like(x)
    sp = c["sp"]
    E = sp.n_elements
    if form == "packed":
        c["op"].apply(x, y)
    else:
        prev = lib.sfem_gb300_set_laplacian_kernel(1 if form == "warp_element_matrix" else -1)
        try:
            capi.check(lib.cu_laplacian_apply(sp.element_type, capi.i64(E), sp.elements_ptrs.ptr, capi.i64(E),
                                              capi.vp(c["op"].fff), capi.FLOAT64, capi.vp(x), capi.vp(y), None),
                       "cu_laplacian_apply")
        finally:
            lib.sfem_gb300_set_laplacian_kernel(prev)
    torch.cuda.synchronize()
    assert lib.sfem_gb300_laplacian_status() == 0
    err = np.abs(y.cpu().numpy() - c["ref"]) / c["scale"]
    assert err.max() < RTOL64, (form, err.max())


@pytest.mark.parametrize("form", ["packed_element_matrix", "packed_stencil", "soa_default"])
def test_cube48_fp32_apply(cuda, cube48, form):
    """FP32 on the 48^3 L = 4 mesh: the benchmark's step (packed tiles, stencil kernel),
    the packed element-matrix kernel and cu_laplacian_apply's float default (stencil
    kernel from the SoA rows)."""
    import torch

    c = cube48
    lib = capi.load()
    x = torch.from_numpy(c["x"]).float().to(cuda)
    y = torch.zeros_like(x)
    sp = c["sp"]
    E = sp.n_elements
    prev = lib.sfem_gb300_set_laplacian_kernel(3 if form == "packed_element_matrix" else -1)
    try:
        if form.startswith("packed"):
            c["op"].apply(x, y)
        else:
            capi.check(lib.cu_laplacian_apply(sp.element_type, capi.i64(E), sp.elements_ptrs.ptr, capi.i64(E),
                                              capi.vp(c["op"].fff), capi.FLOAT32, capi.vp(x), capi.vp(y), None),
                       "cu_laplacian_apply")
        torch.cuda.synchronize()
    finally:
        lib.sfem_gb300_set_laplacian_kernel(prev)
    assert lib.sfem_gb300_laplacian_status() == 0
    err = np.abs(y.double().cpu().numpy() - c["ref"]) / c["scale"]
    assert err.max() < RTOL32, (form, err.max())


def test_cantilever_elasticity_apply(cuda):
    """FP64 and FP32 (the default tcgen05 3xTF32 kernel at L = 4) elasticity applies on
    the 64 x 16 x 16 L = 4 cantilever against the oracle."""
    import ctypes

    import torch

    L = 4
    m = SSMesh(64, 16, 16, L, box=((0, 4), (0, 1), (0, 1)), perturb=0.0, seed=0)
    sp = SSMeshDevice(m, L, device=cuda)
    el = m.elements(L)
    adj, det = O.adjugate_fill(el[m.macro_corner_lidx(L)], m.points)
    adj_d = torch.from_numpy(adj.T.copy()).to(cuda)
    det_d = torch.from_numpy(det.copy()).to(cuda)
    n = m.n_nodes(L)
    u = np.random.default_rng(2).standard_normal(3 * n)
    ref = O.linear_elasticity_apply(L, el, adj, det, MU, LAM, u)
    scale = O.linear_elasticity_row_scale(L, el, adj, det, MU, LAM, u)
    lib = capi.load()
    E = m.n_elements
    for dt, rt, tol in ((torch.float64, capi.FLOAT64, RTOL64), (torch.float32, capi.FLOAT32, RTOL32)):
        ud = torch.from_numpy(u).to(dt).to(cuda)
        yd = torch.zeros_like(ud)
        capi.check(lib.sfem_gb300_linear_elasticity_apply(sp.element_type, capi.i64(E), sp.elements_ptrs.ptr,
                                                          capi.i64(E), capi.vp(adj_d), capi.vp(det_d),
                                                          ctypes.c_double(MU), ctypes.c_double(LAM), rt, capi.vp(ud),
                                                          capi.vp(yd), None), "elasticity apply")
        torch.cuda.synchronize()
        err = np.abs(yd.double().cpu().numpy() - ref) / scale
        assert err.max() < tol, (dt, err.max())
    assert lib.sfem_gb300_elasticity_status() == 0
