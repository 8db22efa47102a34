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


@pytest.mark.parametrize("L,n", [(2, (3, 2, 2)), (3, (2, 3, 2)), (4, (3, 3, 2)), (5, (2, 1, 2)), (6, (2, 2, 1)),
                                 (8, (1, 2, 2)), (12, (1, 1, 2)), (16, (2, 1, 1))])
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


@pytest.mark.parametrize("L,n", [(2, (3, 2, 2)), (3, (3, 2, 2)), (4, (3, 2, 2)), (6, (2, 2, 1)), (7, (1, 2, 1)),
                                 (8, (1, 2, 2)), (16, (1, 1, 2))])
def test_sshex8_laplacian_apply_fp32(cuda, L, n):
    """The float apply with the default kernel of each level (L = 6, 8: warp kernel;
    7, 16: CTA per element)."""
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


@pytest.mark.parametrize("variant", [0, 1, 2, 3, 4, 6, 7, 8])
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


@pytest.mark.parametrize("variant", [1, -1, 8])
@pytest.mark.parametrize("L", [2, 3, 4])
@pytest.mark.parametrize("n", [(5, 4, 3), (1, 1, 1), (8, 5, 3)])
@pytest.mark.parametrize("aligned", [True, False])
def test_sshex8_laplacian_fp64_kernels(cuda, variant, L, n, aligned):
    """FP64 at L = 2, 3, 4: the default kernel (-1), the node-centric stencil kernel (8)
    and the warp element-matrix kernel (1), on ragged tiles (60 = 32 + 28, 1, 120 = 3 x
    32 + 24) with connectivity rows 16-byte aligned or not; 1e-13 of the row scale."""
    import torch

    m = SSMesh(*n, L, perturb=0.1, seed=12)
    el = m.elements(L)
    E = m.n_elements
    fff_aos = O.fff_fill(el[m.macro_corner_lidx(L)], m.points)
    stride = E if aligned else E + 1
    fbuf = torch.zeros((6, stride), dtype=torch.float32, device=cuda)
    fbuf[:, :E] = torch.from_numpy(fff_aos.T.copy()).to(cuda)
    buf = torch.zeros((el.shape[0], stride), dtype=torch.int32, device=cuda)
    buf[:, :E] = torch.from_numpy(el).to(cuda)
    rows = capi.DevicePtrArray(buf)
    rng = np.random.default_rng(13)
    x, y0 = rng.standard_normal(m.n_nodes(L)), rng.standard_normal(m.n_nodes(L))
    ref = O.sshex8_laplacian_stencil_apply(L, el, fff_aos, x, out=y0.copy())
    xd, yd = torch.from_numpy(x).to(cuda), torch.from_numpy(y0).to(cuda)
    lib = capi.load()
    prev = lib.sfem_gb300_set_laplacian_kernel(variant)
    try:
        capi.check(lib.cu_laplacian_apply(capi.SSHEX8(L), capi.i64(E), rows.ptr, capi.i64(stride), capi.vp(fbuf),
                                          capi.FLOAT64, capi.vp(xd), capi.vp(yd), None), "apply")
        torch.cuda.synchronize()
    finally:
        lib.sfem_gb300_set_laplacian_kernel(prev)
    scale = _row_scale_lap(L, el, fff_aos, x) + np.abs(y0)
    err = np.abs(yd.cpu().numpy() - ref) / scale
    assert err.max() < RTOL64, (variant, n, aligned, err.max())


@pytest.mark.parametrize("form", ["fp32_em", "fp32_stencil", "fp64_stencil"])
@pytest.mark.parametrize("n", [(5, 4, 3), (9, 8, 7), (1, 1, 1), (36, 36, 36), (2, 16, 1), (3, 11, 1)])
@pytest.mark.parametrize("aligned", [True, False])
@pytest.mark.parametrize("L", [4, 3])
def test_sshex8_laplacian_packed(cuda, form, n, aligned, L):
    """Packed tiles (L = 4 and 3): pack from SoA rows (row stride E or E + 1) and apply
    with the FP32 stencil kernel (default), the FP32 element-matrix kernel (L = 4, any
    other forced variant) or FP64 (stencil kernel); element counts 60 (32 + 28: a ragged
    last tile), 504, 1, 46,656, 32 (one full tile) and 33 (a last tile of one element)."""
    import torch

    if form == "fp32_em" and L != 4:
        pytest.skip("the element-matrix packed kernel serves L = 4")
    m = SSMesh(*n, L, perturb=0.1, seed=6)
    el = m.elements(L)
    E = m.n_elements
    fff_aos = O.fff_fill(el[m.macro_corner_lidx(L)], m.points)
    stride = E if aligned else E + 1
    fbuf = torch.zeros((6, stride), dtype=torch.float32, device=cuda)
    fbuf[:, :E] = torch.from_numpy(fff_aos.T.copy()).to(cuda)
    buf = torch.zeros((el.shape[0], stride), dtype=torch.int32, device=cuda)
    buf[:, :E] = torch.from_numpy(el).to(cuda)
    rows = capi.DevicePtrArray(buf)
    lib = capi.load()
    nbytes = lib.sfem_gb300_sshex8_packed_bytes(capi.SSHEX8(L), capi.i64(E))
    nxe = el.shape[0]
    assert nbytes == (E + 31) // 32 * 32 * (nxe + 6) * 4
    packed = torch.empty(nbytes // 4, dtype=torch.int32, device=cuda)
    capi.check(lib.sfem_gb300_sshex8_pack(capi.SSHEX8(L), capi.i64(E), rows.ptr, capi.i64(stride), capi.vp(fbuf),
                                          capi.vp(packed), None), "pack")
    # layout: tile t = [node][el] ids, then [6][el] metric bits; padding node 0, metric 0
    blk = packed.view(-1, 32 * (nxe + 6)).cpu().numpy()
    ids = blk[:, :32 * nxe].reshape(-1, nxe, 32).transpose(0, 2, 1).reshape(-1, nxe)
    assert np.array_equal(ids[:E], el.T) and not ids[E:].any()
    met = blk[:, 32 * nxe:].reshape(-1, 6, 32).transpose(0, 2, 1).reshape(-1, 6).view(np.float32)
    assert np.array_equal(met[:E], fff_aos.astype(np.float32)) and not met[E:].any()
    x = np.random.default_rng(7).standard_normal(m.n_nodes(L))
    y0 = np.random.default_rng(8).standard_normal(m.n_nodes(L))
    ref = O.sshex8_laplacian_apply(L, el, fff_aos, x, out=y0.copy())
    dt, rt, tol = (torch.float64, capi.FLOAT64, RTOL64) if form == "fp64_stencil" else (torch.float32, capi.FLOAT32, RTOL32)
    xd = torch.from_numpy(x).to(dt).to(cuda)
    yd = torch.from_numpy(y0).to(dt).to(cuda)
    variant = 3 if form == "fp32_em" else -1
    prev = lib.sfem_gb300_set_laplacian_kernel(variant)
    try:
        capi.check(lib.sfem_gb300_sshex8_laplacian_apply_packed(capi.SSHEX8(L), capi.i64(E), capi.vp(packed),
                                                                rt, capi.vp(xd), capi.vp(yd), None),
                   "apply_packed")
        torch.cuda.synchronize()
    finally:
        lib.sfem_gb300_set_laplacian_kernel(prev)
    assert lib.sfem_gb300_laplacian_status() == 0
    scale = _row_scale_lap(L, el, fff_aos, x) + np.abs(y0)
    err = np.abs(yd.double().cpu().numpy() - ref) / scale
    assert err.max() < tol, (form, n, aligned, err.max())


@pytest.mark.parametrize("form", ["fp32_stencil", "fp32_em", "fp64_stencil"])
def test_tile_wait_gives_up_and_reports(cuda, form):
    """Failure detection without a fault: the first wait on each tile's bulk copy is
    given no polls, so every tile gives up.  Each CTA records the status and drains
    its copy (normal long bound) before it exits; the status is reported once, the
    context stays usable and the next apply is exact."""
    import torch

    L = 4
    m = SSMesh(24, 24, 24, L, perturb=0.1, seed=14)
    sp = SSMeshDevice(m, L)
    el = m.elements(L)
    fff_aos = O.fff_fill(el[m.macro_corner_lidx(L)], m.points)
    op = Laplacian(sp, packed=True).set_fff(torch.from_numpy(fff_aos.T.copy()))
    dt = torch.float64 if form == "fp64_stencil" else torch.float32
    x = torch.from_numpy(np.random.default_rng(15).standard_normal(m.n_nodes(L))).to(dt).to(cuda)
    y = torch.zeros_like(x)
    lib = capi.load()
    assert lib.sfem_gb300_laplacian_status() == 0
    kprev = lib.sfem_gb300_set_laplacian_kernel(3 if form == "fp32_em" else -1)
    try:
        prev = lib.sfem_gb300_set_tile_wait_polls(0)
        try:
            op.apply(x, y)
            torch.cuda.synchronize()
        finally:
            lib.sfem_gb300_set_tile_wait_polls(prev)
        assert lib.sfem_gb300_laplacian_status() == 1  # gave up, drained, reported
        assert lib.sfem_gb300_laplacian_status() == 0  # read and cleared
        y.zero_()
        op.apply(x, y)
        torch.cuda.synchronize()
    finally:
        lib.sfem_gb300_set_laplacian_kernel(kprev)
    assert lib.sfem_gb300_laplacian_status() == 0
    ref = O.sshex8_laplacian_apply(L, el, fff_aos, x.double().cpu().numpy())
    scale = _row_scale_lap(L, el, fff_aos, x.double().cpu().numpy())
    tol = RTOL64 if dt == torch.float64 else RTOL32
    assert (np.abs(y.double().cpu().numpy() - ref) / scale).max() < tol


def test_sshex8_laplacian_packed_operator(cuda):
    """The operator's FP32 and FP64 applies go through the packed blocks."""
    import torch

    L = 4
    m = SSMesh(3, 2, 2, L, perturb=0.1, seed=9)
    sp = SSMeshDevice(m, L)
    el = m.elements(L)
    fff_aos = O.fff_fill(el[m.macro_corner_lidx(L)], m.points)
    op = Laplacian(sp, packed=True).set_fff(torch.from_numpy(fff_aos.T.copy()))
    assert op.packed_blocks is not None
    x = np.random.default_rng(10).standard_normal(m.n_nodes(L))
    ref = O.sshex8_laplacian_apply(L, el, fff_aos, x)
    y32 = torch.zeros(m.n_nodes(L), dtype=torch.float32, device=cuda)
    op.apply(torch.from_numpy(x).float().to(cuda), y32)
    y64 = torch.zeros(m.n_nodes(L), dtype=torch.float64, device=cuda)
    op.apply(torch.from_numpy(x).to(cuda), y64)
    scale = _row_scale_lap(L, el, fff_aos, x)
    assert (np.abs(y32.double().cpu().numpy() - ref) / scale).max() < RTOL32
    assert (np.abs(y64.cpu().numpy() - ref) / scale).max() < RTOL64


def test_sshex8_laplacian_packed_bad_inputs(cuda):
    import torch

    lib = capi.load()
    # packed tiles serve L = 3 and 4 only
    assert lib.sfem_gb300_sshex8_packed_bytes(capi.SSHEX8(2), capi.i64(10)) == -1
    assert lib.sfem_gb300_sshex8_packed_bytes(capi.SSHEX8(5), capi.i64(10)) == -1
    assert lib.sfem_gb300_sshex8_packed_bytes(capi.SSHEX8(3), capi.i64(10)) == 32 * (64 + 6) * 4
    assert lib.sfem_gb300_sshex8_packed_bytes(capi.SSHEX8(4), capi.i64(0)) == 0
    buf = torch.zeros(64, dtype=torch.int32, device=cuda)
    x = torch.zeros(8, dtype=torch.float64, device=cuda)
    # an unknown real type is refused with a message
    assert lib.sfem_gb300_sshex8_laplacian_apply_packed(capi.SSHEX8(4), capi.i64(1), capi.vp(buf), 7,
                                                        capi.vp(x), capi.vp(x), None) == 1
    assert "real type" in capi.last_error()
    # a block array that is not 16-byte aligned is refused before any launch
    assert lib.sfem_gb300_sshex8_laplacian_apply_packed(capi.SSHEX8(4), capi.i64(1), capi.c_void(buf.data_ptr() + 4),
                                                        capi.FLOAT32, capi.vp(x), capi.vp(x), None) == 1
    assert "aligned" in capi.last_error()


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


@pytest.mark.parametrize("L", [2, 3, 4, 5, 16])
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
    assert lib.cu_laplacian_apply(capi.SSHEX8(17), capi.i64(1), sp.elements_ptrs.ptr, capi.i64(1), None,
                                  capi.FLOAT64, capi.vp(y), capi.vp(y), None) == 1
    assert "unsupported" in capi.last_error()
    assert lib.cu_laplacian_apply(capi.SSHEX8(4), capi.i64(1), sp.elements_ptrs.ptr, capi.i64(1), None,
                                  7, capi.vp(y), capi.vp(y), None) == 1


@pytest.mark.parametrize("dtype_name,tol", [("float64", 1e-13), ("float32", 2e-5)])
@pytest.mark.parametrize("L,n", [(1, (3, 2, 2)), (4, (3, 2, 2)), (5, (2, 1, 1)), (8, (1, 2, 1))])
def test_sshex8_laplacian_stored_element_matrices(cuda, dtype_name, tol, L, n):
    """ss:em form: the stored 8 x 8 micro element matrices equal the oracle's, and the
    apply from them equals the oracle apply."""
    import torch

    dt = getattr(torch, dtype_name)
    rt = capi.FLOAT64 if dt == torch.float64 else capi.FLOAT32
    m = SSMesh(*n, L, perturb=0.1, seed=3)
    sp = SSMeshDevice(m, L)
    el = m.elements(L)
    fff_aos = O.fff_fill(el[m.macro_corner_lidx(L)], m.points)
    E = m.n_elements
    fff = torch.from_numpy(fff_aos.T.copy()).to(cuda)
    lib = capi.load()
    em = torch.empty(E * 64, dtype=dt, device=cuda)
    capi.check(lib.sfem_gb300_sshex8_laplacian_element_matrix(capi.SSHEX8(L), capi.i64(E), capi.i64(E), capi.vp(fff),
                                                              rt, capi.vp(em), None), "element matrices")
    ref_em = np.stack([O.laplacian_matrix(fff_aos[e].astype(np.float64) / L).reshape(64) for e in range(E)])
    assert np.abs(em.double().cpu().numpy().reshape(E, 64) - ref_em).max() <= (1e-14 if tol < 1e-10 else 1e-6) * np.abs(ref_em).max()
    x = np.random.default_rng(11).standard_normal(m.n_nodes(L))
    ref = O.sshex8_laplacian_apply(L, el, fff_aos, x) if L > 1 else O.hex8_laplacian_apply(m.hex8_elements(), fff_aos, x)
    y = torch.zeros(m.n_nodes(L), dtype=dt, device=cuda)
    elp = sp.elements_ptrs if L > 1 else capi.DevicePtrArray(torch.from_numpy(np.ascontiguousarray(el)).to(cuda))
    capi.check(lib.sfem_gb300_sshex8_laplacian_apply_em(capi.SSHEX8(L), capi.i64(E), elp.ptr, capi.vp(em), rt,
                                                        capi.vp(torch.from_numpy(x).to(dt).to(cuda)), capi.vp(y), None),
               "apply_em")
    scale = _row_scale_lap(L, el if L > 1 else m.hex8_elements(), fff_aos, x)
    assert (np.abs(y.double().cpu().numpy() - ref) / scale).max() < tol
