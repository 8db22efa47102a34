"""GPU parity of the matrix-free Laplacian (C ABI) against the CPU oracle.

Tolerance: the FP64 apply must match the oracle to 1e-13 relative per entry,
measured against the row scale (|A| |x|)_i so that entries that cancel to
~0 are judged against the size of the terms that produced them.
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


def _row_scale_lap(L, el, fff_aos, x):
    # (|A| |x|) via the oracle applied to |x| with |A| ... approximate by the
    # abs-valued element matrices: use the diag-dominance bound |A||x| <= 2 diag*|x| on
    # a Laplacian (rows sum to zero) -> use A(|x|) + 2 diag |x| as a safe scale
    n = x.size
    ax = O.sshex8_laplacian_apply(L, el, fff_aos, np.abs(x)) if L > 1 else O.hex8_laplacian_apply(el, fff_aos, np.abs(x))
    d = O.laplacian_diag(L if L > 1 else 0, el, fff_aos, n)
    return np.abs(ax) + 2 * d * np.abs(x)


@pytest.mark.parametrize("L,n", [(2, (3, 2, 2)), (3, (2, 3, 2)), (4, (3, 3, 2)), (6, (2, 2, 1)), (8, (1, 2, 2))])
def test_sshex8_laplacian_apply_fp64(cuda, L, n):
    import torch

    m = SSMesh(*n, L, perturb=0.1, seed=L)
    sp = SSMeshDevice(m, L)
    el = m.elements(L)
    fff_aos = O.fff_fill(el[m.macro_corner_lidx(L)], m.points)
    op = Laplacian(sp).set_fff(torch.from_numpy(fff_aos.T.copy()))
    rng = np.random.default_rng(L)
    x = rng.standard_normal(m.n_nodes(L))
    y0 = rng.standard_normal(m.n_nodes(L))
    ref = O.sshex8_laplacian_apply(L, el, fff_aos, x, out=y0.copy())
    xd = torch.from_numpy(x).to(cuda)
    yd = torch.from_numpy(y0).to(cuda)
    op.apply(xd, yd)
    got = yd.cpu().numpy()
    scale = _row_scale_lap(L, el, fff_aos, x) + np.abs(y0)
    err = np.abs(got - ref) / scale
    assert err.max() < RTOL64, err.max()


@pytest.mark.parametrize("L,n", [(2, (3, 2, 2)), (3, (3, 2, 2)), (4, (3, 2, 2)), (6, (2, 2, 1)), (8, (1, 2, 2))])
def test_sshex8_laplacian_apply_fp32(cuda, L, n):
    """The float apply with the default kernel of each level (L = 6, 8: warp kernel)."""
    import torch

    m = SSMesh(*n, L, perturb=0.1, seed=1)
    sp = SSMeshDevice(m, L)
    el = m.elements(L)
    fff_aos = O.fff_fill(el[m.macro_corner_lidx(L)], m.points)
    op = Laplacian(sp).set_fff(torch.from_numpy(fff_aos.T.copy()))
    x = np.random.default_rng(3).standard_normal(m.n_nodes(L))
    ref = O.sshex8_laplacian_apply(L, el, fff_aos, x)
    yd = torch.zeros(m.n_nodes(L), dtype=torch.float32, device=cuda)
    op.apply(torch.from_numpy(x).float().to(cuda), yd)
    scale = _row_scale_lap(L, el, fff_aos, x)
    err = np.abs(yd.double().cpu().numpy() - ref) / scale
    assert err.max() < RTOL32, err.max()


@pytest.mark.parametrize("variant", [0, 1, 2, 3, 4, 6, 7])
@pytest.mark.parametrize("L", [2, 3, 4])
@pytest.mark.parametrize("aligned", [True, False])
def test_sshex8_laplacian_fp32_kernels(cuda, variant, L, aligned):
    """Every float kernel on a mesh whose element count is not a tile multiple (60 =
    32 + 28), with connectivity rows 16-byte aligned or not (row stride E + 1)."""
    import torch

    m = SSMesh(5, 4, 3, L, perturb=0.1, seed=2)
    el = m.elements(L)
    E = m.n_elements
    fff_aos = O.fff_fill(el[m.macro_corner_lidx(L)], m.points)
    fff = torch.from_numpy(fff_aos.T.copy()).to(cuda)
    stride = E if aligned else E + 1
    buf = torch.zeros((el.shape[0], stride), dtype=torch.int32, device=cuda)
    buf[:, :E] = torch.from_numpy(el).to(cuda)
    rows = capi.DevicePtrArray(buf)
    x = np.random.default_rng(4).standard_normal(m.n_nodes(L))
    y0 = np.random.default_rng(5).standard_normal(m.n_nodes(L))
    ref = O.sshex8_laplacian_apply(L, el, fff_aos, x, out=y0.copy())
    xd = torch.from_numpy(x).float().to(cuda)
    yd = torch.from_numpy(y0).float().to(cuda)
    lib = capi.load()
    prev = lib.sfem_gb300_set_laplacian_kernel(variant)
    try:
        capi.check(lib.cu_laplacian_apply(capi.SSHEX8(L), capi.i64(E), rows.ptr, capi.i64(E), capi.vp(fff),
                                          capi.FLOAT32, capi.vp(xd), capi.vp(yd), None), "apply")
        torch.cuda.synchronize()
    finally:
        lib.sfem_gb300_set_laplacian_kernel(prev)
    scale = _row_scale_lap(L, el, fff_aos, x) + np.abs(y0)
    err = np.abs(yd.double().cpu().numpy() - ref) / scale
    assert err.max() < RTOL32, (variant, L, aligned, err.max())


def test_hex8_laplacian_apply_and_diag(cuda):
    import torch

    m = SSMesh(5, 4, 3, 1, perturb=0.2, seed=5)
    sp = SSMeshDevice(m, 1)
    el = m.hex8_elements()
    fff_aos = O.fff_fill(el, m.points)
    op = Laplacian(sp).set_fff(torch.from_numpy(fff_aos.T.copy()))
    x = np.random.default_rng(0).standard_normal(m.n_nodes(1))
    ref = O.hex8_laplacian_apply(el, fff_aos, x)
    yd = torch.zeros(m.n_nodes(1), dtype=torch.float64, device=cuda)
    op.apply(torch.from_numpy(x).to(cuda), yd)
    scale = _row_scale_lap(1, el, fff_aos, x)
    assert (np.abs(yd.cpu().numpy() - ref) / scale).max() < RTOL64
    d_ref = O.laplacian_diag(0, el, fff_aos, m.n_nodes(1))
    dd = torch.zeros(m.n_nodes(1), dtype=torch.float64, device=cuda)
    op.hessian_diag(dd)
    assert np.abs(dd.cpu().numpy() - d_ref).max() <= 1e-13 * np.abs(d_ref).max()


@pytest.mark.parametrize("L", [2, 3, 4])
def test_sshex8_laplacian_diag(cuda, L):
    import torch

    m = SSMesh(2, 3, 2, L, perturb=0.1, seed=2)
    sp = SSMeshDevice(m, L)
    el = m.elements(L)
    fff_aos = O.fff_fill(el[m.macro_corner_lidx(L)], m.points)
    op = Laplacian(sp).set_fff(torch.from_numpy(fff_aos.T.copy()))
    d_ref = O.laplacian_diag(L, el, fff_aos, m.n_nodes(L))
    dd = torch.zeros(m.n_nodes(L), dtype=torch.float64, device=cuda)
    op.hessian_diag(dd)
    assert np.abs(dd.cpu().numpy() - d_ref).max() <= 1e-13 * np.abs(d_ref).max()


def test_fff_fill_matches_oracle(cuda):
    import torch

    m = SSMesh(4, 3, 3, 4, perturb=0.15, seed=7)
    sp = SSMeshDevice(m, 4)
    op = Laplacian(sp).initialize()
    el = m.elements(4)
    ref = O.fff_fill(el[m.macro_corner_lidx(4)], m.points)
    got = op.fff.cpu().numpy().T
    # computed in double from float coordinates then rounded: at most 1 float ulp apart
    assert np.all(np.abs(got - ref) <= 2.5e-7 * np.abs(ref).max())


def test_empty_and_bad_inputs(cuda):
    import torch

    m = SSMesh(1, 1, 1, 4)
    sp = SSMeshDevice(m, 4)
    lib = capi.load()
    y = torch.zeros(m.n_nodes(), dtype=torch.float64, device=cuda)
    # zero elements: success, no work
    assert lib.cu_laplacian_apply(capi.SSHEX8(4), capi.i64(0), sp.elements_ptrs.ptr, capi.i64(0), None,
                                  capi.FLOAT64, capi.vp(y), capi.vp(y), None) == 0
    # unsupported level: failure with a message, no abort
    assert lib.cu_laplacian_apply(capi.SSHEX8(5), capi.i64(1), sp.elements_ptrs.ptr, capi.i64(1), None,
                                  capi.FLOAT64, capi.vp(y), capi.vp(y), None) == 1
    assert "unsupported" in capi.last_error()
    assert lib.cu_laplacian_apply(capi.SSHEX8(4), capi.i64(1), sp.elements_ptrs.ptr, capi.i64(1), None,
                                  7, capi.vp(y), capi.vp(y), None) == 1
