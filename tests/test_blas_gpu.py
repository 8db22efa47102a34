"""GPU vector kernels (BLAS<T> seam) against numpy."""

import ctypes

import numpy as np
import pytest

from sfem_gb300 import capi

pytestmark = pytest.mark.gpu
D = ctypes.c_double


@pytest.fixture()
def ws(cuda):
    import torch

    w = torch.zeros(capi.load().sfem_gb300_reduce_workspace_size(), dtype=torch.uint8, device=cuda)
    return w


@pytest.mark.parametrize("n", [0, 1, 31, 257, 100_000, 3_000_001])
@pytest.mark.parametrize("dt", ["f64", "f32"])
def test_dot_norm_deterministic(cuda, ws, n, dt):
    import torch

    lib = capi.load()
    tdt = torch.float64 if dt == "f64" else torch.float32
    rt = capi.FLOAT64 if dt == "f64" else capi.FLOAT32
    g = torch.Generator(device=cuda).manual_seed(n)
    x = torch.randn(n, dtype=tdt, device=cuda, generator=g)
    y = torch.randn(n, dtype=tdt, device=cuda, generator=g)
    res = torch.zeros(4, dtype=torch.float64, device=cuda)
    capi.check(lib.sfem_gb300_dot(rt, capi.i64(n), capi.vp(x), capi.vp(y), capi.vp(ws), capi.vp(res), None), "dot")
    capi.check(lib.sfem_gb300_dot(rt, capi.i64(n), capi.vp(x), capi.vp(y), capi.vp(ws),
                                  capi.c_void(res.data_ptr() + 8), None), "dot")
    capi.check(lib.sfem_gb300_norm2(rt, capi.i64(n), capi.vp(x), capi.vp(ws), capi.c_void(res.data_ptr() + 16), None),
               "norm2")
    r = res.cpu().numpy()
    ref = float(x.double().cpu().numpy() @ y.double().cpu().numpy())
    nrm = float(np.linalg.norm(x.double().cpu().numpy()))
    tol = 1e-12 if dt == "f64" else 1e-5
    assert r[0] == r[1]  # bitwise reproducible
    assert abs(r[0] - ref) <= tol * max(1.0, np.sqrt(n)) * (1 + abs(ref))
    assert abs(r[2] - nrm) <= tol * (1 + nrm)


def test_elementwise(cuda):
    import torch

    lib = capi.load()
    n = 12345
    g = torch.Generator(device=cuda).manual_seed(0)
    x = torch.randn(n, dtype=torch.float64, device=cuda, generator=g)
    y = torch.randn(n, dtype=torch.float64, device=cuda, generator=g)
    z = torch.zeros(n, dtype=torch.float64, device=cuda)
    xn, yn = x.cpu().numpy(), y.cpu().numpy()
    yy = y.clone()
    capi.check(lib.sfem_gb300_axpby(capi.FLOAT64, capi.i64(n), D(2.0), capi.vp(x), D(-0.5), capi.vp(yy), None), "")
    assert np.allclose(yy.cpu().numpy(), 2 * xn - 0.5 * yn, rtol=1e-15, atol=1e-15)
    capi.check(lib.sfem_gb300_zaxpby(capi.FLOAT64, capi.i64(n), D(1.5), capi.vp(x), D(3.0), capi.vp(y), capi.vp(z),
                                     None), "")
    assert np.allclose(z.cpu().numpy(), 1.5 * xn + 3 * yn, rtol=1e-15, atol=1e-14)
    zz = z.clone()
    capi.check(lib.sfem_gb300_xypaz(capi.FLOAT64, capi.i64(n), capi.vp(x), capi.vp(y), D(0.5), capi.vp(zz), None), "")
    assert np.allclose(zz.cpu().numpy(), xn * yn + 0.5 * z.cpu().numpy(), rtol=1e-14, atol=1e-14)
    w = x.clone()
    w[::7] = 0
    capi.check(lib.sfem_gb300_reciprocal(capi.FLOAT64, capi.i64(n), D(0.3), capi.vp(w), None), "")
    wn = x.cpu().numpy().copy()
    wn[::7] = 0
    expect = np.where(wn != 0, 0.3 / np.where(wn != 0, wn, 1), 0)
    assert np.allclose(w.cpu().numpy(), expect, rtol=1e-15)
    # Chebyshev update
    p = y.clone()
    xx = x.clone()
    rhs = z.clone()
    capi.check(lib.sfem_gb300_chebyshev_update(capi.FLOAT64, capi.i64(n), D(0.7), D(0.2), None, capi.vp(rhs),
                                               capi.vp(y), capi.vp(p), capi.vp(xx), None), "")
    pn = 0.2 * yn - z.cpu().numpy() + yn
    assert np.allclose(p.cpu().numpy(), pn, rtol=1e-14, atol=1e-14)
    assert np.allclose(xx.cpu().numpy(), xn - 0.7 * pn, rtol=1e-14, atol=1e-14)
    # Jacobi-scaled variant, beta = 0 ignores the old p (even if it holds NaN)
    inv = torch.rand(n, dtype=torch.float64, device=cuda, generator=g) + 0.5
    p2 = torch.full_like(y, float("nan"))
    x2 = x.clone()
    capi.check(lib.sfem_gb300_chebyshev_update(capi.FLOAT64, capi.i64(n), D(0.7), D(0.0), capi.vp(inv), capi.vp(rhs),
                                               capi.vp(y), capi.vp(p2), capi.vp(x2), None), "")
    pn2 = inv.cpu().numpy() * (yn - z.cpu().numpy())
    assert np.allclose(p2.cpu().numpy(), pn2, rtol=1e-14, atol=1e-14)
    assert np.allclose(x2.cpu().numpy(), xn - 0.7 * pn2, rtol=1e-14, atol=1e-14)
    # conversions
    f = torch.zeros(n, dtype=torch.float32, device=cuda)
    capi.check(lib.sfem_gb300_convert(capi.i64(n), capi.FLOAT64, capi.vp(x), capi.FLOAT32, capi.vp(f), None), "")
    assert torch.equal(f, x.float())
    acc = y.clone()
    capi.check(lib.sfem_gb300_axpy_f32_to_f64(capi.i64(n), D(2.0), capi.vp(f), capi.vp(acc), None), "")
    assert np.allclose(acc.cpu().numpy(), yn + 2 * f.double().cpu().numpy(), rtol=1e-15, atol=1e-15)


def test_cg_fused_updates(cuda, ws):
    import torch

    lib = capi.load()
    n = 50_001
    g = torch.Generator(device=cuda).manual_seed(1)
    p, Ap, x, r = (torch.randn(n, dtype=torch.float64, device=cuda, generator=g) for _ in range(4))
    sc = torch.tensor([2.0, 4.0, 0.0], dtype=torch.float64, device=cuda)  # alpha = 0.5
    xr, rr = x.cpu().numpy() + 0.5 * p.cpu().numpy(), r.cpu().numpy() - 0.5 * Ap.cpu().numpy()
    capi.check(lib.sfem_gb300_cg_update_x_r(capi.FLOAT64, capi.i64(n), capi.vp(sc), capi.c_void(sc.data_ptr() + 8),
                                            capi.vp(p), capi.vp(Ap), capi.vp(x), capi.vp(r), capi.vp(ws),
                                            capi.c_void(sc.data_ptr() + 16), None), "")
    assert np.allclose(x.cpu().numpy(), xr, rtol=1e-15, atol=1e-15)
    assert np.allclose(r.cpu().numpy(), rr, rtol=1e-15, atol=1e-15)
    assert abs(sc[2].item() - rr @ rr) <= 1e-11 * (rr @ rr)
    z = torch.randn(n, dtype=torch.float64, device=cuda, generator=g)
    pp = p.clone()
    capi.check(lib.sfem_gb300_cg_update_p(capi.FLOAT64, capi.i64(n), capi.vp(sc), capi.c_void(sc.data_ptr() + 8),
                                          None, capi.vp(z), capi.vp(pp), None), "")
    assert np.allclose(pp.cpu().numpy(), z.cpu().numpy() + 0.5 * p.cpu().numpy(), rtol=1e-15, atol=1e-15)
    # flexible (Polak-Ribiere) form: beta = (2 - 1) / 4
    sub = torch.tensor([1.0], dtype=torch.float64, device=cuda)
    pf = p.clone()
    capi.check(lib.sfem_gb300_cg_update_p(capi.FLOAT64, capi.i64(n), capi.vp(sc), capi.c_void(sc.data_ptr() + 8),
                                          capi.vp(sub), capi.vp(z), capi.vp(pf), None), "")
    assert np.allclose(pf.cpu().numpy(), z.cpu().numpy() + 0.25 * p.cpu().numpy(), rtol=1e-15, atol=1e-15)


def test_dirichlet_kernels(cuda):
    import torch

    lib = capi.load()
    nodes = torch.tensor([0, 5, 9], dtype=torch.int32, device=cuda)
    src = torch.arange(30, dtype=torch.float64, device=cuda)
    dst = torch.zeros(30, dtype=torch.float64, device=cuda)
    capi.check(lib.sfem_gb300_constraint_nodes_copy(capi.FLOAT64, capi.i64(3), capi.vp(nodes), 3, 1, capi.vp(src),
                                                    capi.vp(dst), None), "")
    assert dst.cpu().numpy()[[1, 16, 28]].tolist() == [1, 16, 28] and dst.sum().item() == 45
    capi.check(lib.sfem_gb300_constraint_nodes_to_value(capi.FLOAT64, capi.i64(3), capi.vp(nodes), 1, 0, D(7.0),
                                                        capi.vp(dst), None), "")
    assert dst.cpu().numpy()[[0, 5, 9]].tolist() == [7, 7, 7]


def test_random_uniform_matches_hash(cuda):
    import torch

    from oracle.solvers import random_uniform

    n = 100_003
    for dt, rt in ((torch.float64, capi.FLOAT64), (torch.float32, capi.FLOAT32)):
        x = torch.zeros(n, dtype=dt, device=cuda)
        capi.check(capi.load().sfem_gb300_random_uniform(rt, capi.i64(n), ctypes.c_ulonglong(0x5EED5EED), capi.vp(x),
                                                         None), "random")
        ref = random_uniform(n, 0x5EED5EED)
        assert np.array_equal(x.cpu().numpy(), ref.astype(x.cpu().numpy().dtype))
