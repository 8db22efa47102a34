"""GPU parity of the multigrid transfer operators (prolongation / restriction)."""

import numpy as np
import pytest

import oracle as O
from sfem_gb300 import capi
from sfem_gb300.mesh import SSMesh

pytestmark = pytest.mark.gpu


def _dev(a, cuda):
    import torch

    return torch.from_numpy(np.ascontiguousarray(a)).to(cuda)


@pytest.mark.parametrize("L,lc,vec", [(4, 2, 1), (4, 1, 1), (2, 1, 1), (8, 4, 1), (4, 2, 3), (3, 1, 1), (6, 3, 3)])
def test_prolongate_restrict(cuda, L, lc, vec):
    import torch

    m = SSMesh(3, 2, 2, L, perturb=0.1, seed=1)
    ef, ec = m.elements(L), m.elements(lc)
    nf, nc = m.n_nodes(L), m.n_nodes(lc)
    ef_d, ec_d = _dev(ef, cuda), _dev(ec, cuda)
    pf, pc = capi.DevicePtrArray(ef_d), capi.DevicePtrArray(ec_d)
    lib = capi.load()
    rng = np.random.default_rng(L * 10 + lc)
    xc = rng.standard_normal(nc * vec)
    ref = O.prolongate(lc, ec, L, ef, vec, xc, nf)
    out = torch.zeros(nf * vec, dtype=torch.float64, device=cuda)
    xc_d = _dev(xc, cuda)
    capi.check(lib.sfem_gb300_sshex8_prolongate(capi.i64(m.n_elements), lc, pc.ptr, L, pf.ptr, vec, capi.FLOAT64,
                                                capi.vp(xc_d), capi.vp(out), None), "prolongate")
    assert np.abs(out.cpu().numpy() - ref).max() <= 1e-14 * np.abs(ref).max()

    cnt = O.incidence_count(L, ef, nf)
    cnt_d = torch.zeros(nf, dtype=torch.int16, device=cuda)
    capi.check(lib.sfem_gb300_sshex8_element_node_incidence_count(L, capi.i64(m.n_elements), pf.ptr, capi.vp(cnt_d),
                                                                  None), "count")
    assert np.array_equal(cnt_d.cpu().numpy().view(np.uint16), cnt)
    xf = rng.standard_normal(nf * vec)
    ref_r = O.restrict(L, ef, cnt, lc, ec, vec, xf, nc)
    out_r = torch.zeros(nc * vec, dtype=torch.float64, device=cuda)
    xf_d = _dev(xf, cuda)
    capi.check(lib.sfem_gb300_sshex8_restrict(capi.i64(m.n_elements), L, pf.ptr, capi.vp(cnt_d), lc, pc.ptr, vec,
                                              capi.FLOAT64, capi.vp(xf_d), capi.vp(out_r), None), "restrict")
    assert np.abs(out_r.cpu().numpy() - ref_r).max() <= 1e-13 * np.abs(ref_r).max()
    # R = P^T: (R xf, xc) == (xf, P xc)
    lhs = float(out_r.cpu().numpy() @ xc)
    rhs = float(xf @ out.cpu().numpy())
    assert abs(lhs - rhs) <= 1e-12 * (abs(lhs) + abs(rhs))


def test_prolongation_preserves_constants(cuda):
    """Known answer (frontend/tests/sfem_SemiStructuredMeshTest.cpp:66-117): P 1 = 1 at L=8."""
    import torch

    m = SSMesh(2, 2, 2, 8)
    lib = capi.load()
    for lc in (4, 2, 1):
        ef_d, ec_d = _dev(m.elements(8), cuda), _dev(m.elements(lc), cuda)
        pf, pc = capi.DevicePtrArray(ef_d), capi.DevicePtrArray(ec_d)
        out = torch.zeros(m.n_nodes(8), dtype=torch.float64, device=cuda)
        ones = torch.ones(m.n_nodes(lc), dtype=torch.float64, device=cuda)
        capi.check(lib.sfem_gb300_sshex8_prolongate(capi.i64(m.n_elements), lc, pc.ptr, 8, pf.ptr, 1, capi.FLOAT64,
                                                    capi.vp(ones), capi.vp(out), None), "prolongate")
        assert torch.allclose(out, torch.ones_like(out), atol=1e-14)


def test_transfer_rejects_non_nested(cuda):
    import torch

    m = SSMesh(1, 1, 1, 4)
    lib = capi.load()
    e = capi.DevicePtrArray(_dev(m.elements(4), cuda))
    y = torch.zeros(10, dtype=torch.float64, device=cuda)
    assert lib.sfem_gb300_sshex8_prolongate(capi.i64(1), 3, e.ptr, 4, e.ptr, 1, capi.FLOAT64, capi.vp(y), capi.vp(y),
                                            None) == 1
    assert "nested" in capi.last_error()
