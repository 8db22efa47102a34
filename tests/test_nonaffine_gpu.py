"""The non-affine sshex8 Laplacian on the GPU (sfem_gb300_sshex8_laplacian_apply_nonaffine)
against the oracle restatement of the reference's sshex8_laplacian_apply
(operators/sshex8/sshex8_laplacian.cpp:39-182), itself pinned to the reference's output by
tests/golden/sshex8_nonaffine.npz.  Perturbed macro meshes (general trilinear hexes),
accumulate semantics (y += A x on a nonzero y); tolerance relative to max |A x|: FP64
1e-13, FP32 2e-5."""

import numpy as np
import pytest

import oracle as O
from sfem_gb300 import capi
from sfem_gb300.mesh import SSMesh

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dtype", ["float64", "float32"])
@pytest.mark.parametrize("L,n", [(1, (3, 2, 2)), (2, (3, 2, 2)), (3, (2, 3, 2)), (4, (3, 2, 2)), (5, (2, 1, 2)),
                                 (8, (1, 1, 2)), (4, (7, 6, 5))])
def test_nonaffine_apply_matches_oracle(cuda, L, n, dtype):
    import torch

    m = SSMesh(*n, L, perturb=0.2, seed=7)
    el = m.elements(L)
    E = m.n_elements
    rows = capi.DevicePtrArray(torch.from_numpy(el.astype(np.int32)).to(cuda))
    pts = torch.from_numpy(np.ascontiguousarray(m.points, dtype=np.float32)).to(cuda)
    rng = np.random.default_rng(8)
    x, y0 = rng.standard_normal(m.n_nodes(L)), rng.standard_normal(m.n_nodes(L))
    ref = O.sshex8_laplacian_apply_nonaffine(L, el, m.points, x, out=y0.copy())
    dt = getattr(torch, dtype)
    rt = capi.FLOAT64 if dtype == "float64" else capi.FLOAT32
    xd = torch.from_numpy(x).to(dt).to(cuda)
    yd = torch.from_numpy(y0).to(dt).to(cuda)
    capi.check(capi.load().sfem_gb300_sshex8_laplacian_apply_nonaffine(
        capi.SSHEX8(L), capi.i64(E), rows.ptr, capi.vp(pts[0]), capi.vp(pts[1]), capi.vp(pts[2]), rt, capi.vp(xd),
        capi.vp(yd), None), "apply_nonaffine")
    torch.cuda.synchronize()
    err = np.abs(yd.double().cpu().numpy() - ref).max() / np.abs(ref - y0).max()
    assert err < (1e-13 if dtype == "float64" else 2e-5), (L, n, dtype, err)


def test_nonaffine_apply_bad_inputs(cuda):
    import torch

    lib = capi.load()
    x = torch.zeros(8, dtype=torch.float64, device=cuda)
    assert lib.sfem_gb300_sshex8_laplacian_apply_nonaffine(capi.SSHEX8(17), capi.i64(1), None, None, None, None,
                                                          capi.FLOAT64, capi.vp(x), capi.vp(x), None) == 1
    assert "sshex8" in capi.last_error()
    assert lib.sfem_gb300_sshex8_laplacian_apply_nonaffine(capi.SSHEX8(2), capi.i64(1), None, None, None, None, 7,
                                                          capi.vp(x), capi.vp(x), None) == 1
    assert "real type" in capi.last_error()
    # no elements: nothing to do
    assert lib.sfem_gb300_sshex8_laplacian_apply_nonaffine(capi.SSHEX8(2), capi.i64(0), None, None, None, None,
                                                          capi.FLOAT64, capi.vp(x), capi.vp(x), None) == 0
