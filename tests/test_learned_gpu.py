"""Learned-smoother kernels (BF16 storage, FP32 arithmetic) against the CPU oracle loop nests."""

import ctypes

import numpy as np
import pytest

import oracle as O
from sfem_gb300 import capi

pytestmark = pytest.mark.gpu


def _bf16(a, cuda):
    import torch

    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).to(cuda).to(torch.bfloat16)


def _f(t):
    return t.float().cpu().numpy()


@pytest.mark.parametrize("cin,cout,relu", [(1, 16, 1), (16, 16, 1), (16, 1, 0)])
def test_patchconv_forward_and_gradients(cuda, cin, cout, relu):
    import torch

    rng = np.random.default_rng(cin * 100 + cout)
    P = 37
    x = _bf16(rng.standard_normal((P, 125, cin)), cuda)
    W = _bf16(rng.standard_normal((cout, cin, 27)) / np.sqrt(27 * cin), cuda)
    lib = capi.load()
    y = torch.zeros((P, 125, cout), dtype=torch.bfloat16, device=cuda)
    capi.check(lib.sfem_gb300_patchconv_forward(capi.i64(P), cin, cout, capi.vp(x), capi.vp(W), relu, capi.vp(y),
                                                None), "forward")
    ref = O.patchconv_forward(P, cin, cout, _f(x), _f(W), relu).reshape(P, 125, cout)
    # outputs are rounded to BF16 (8 significant bits)
    assert np.abs(_f(y) - ref).max() <= 1e-2 * np.abs(ref).max()
    g = _bf16(rng.standard_normal((P, 125, cout)), cuda)
    gin = torch.zeros((P, 125, cin), dtype=torch.bfloat16, device=cuda)
    act = x if cin == 16 else None
    capi.check(lib.sfem_gb300_patchconv_backward_data(capi.i64(P), cin, cout, capi.vp(g), capi.vp(W), capi.vp(act),
                                                      capi.vp(gin), None), "backward data")
    ref_gin = O.patchconv_backward_data(P, cin, cout, _f(g), _f(W), _f(act) if act is not None else None)
    assert np.abs(_f(gin).reshape(-1) - ref_gin).max() <= 1e-2 * np.abs(ref_gin).max()
    dW = torch.zeros(cout * cin * 27, dtype=torch.float32, device=cuda)
    capi.check(lib.sfem_gb300_patchconv_backward_weights(capi.i64(P), cin, cout, capi.vp(g), capi.vp(x), capi.vp(dW),
                                                         None), "backward weights")
    ref_dW = O.patchconv_backward_weights(P, cin, cout, _f(g), _f(x))
    # FP32 accumulation of exact BF16 products
    assert np.abs(dW.cpu().numpy() - ref_dW).max() <= 1e-4 * np.abs(ref_dW).max()


def test_adam_and_mse(cuda):
    import torch

    lib = capi.load()
    n = 1000
    y = torch.randn(n, device=cuda).to(torch.bfloat16)
    t = torch.randn(n, device=cuda).to(torch.bfloat16)
    gy = torch.zeros(n, dtype=torch.bfloat16, device=cuda)
    loss = torch.zeros(1, dtype=torch.float32, device=cuda)
    capi.check(lib.sfem_gb300_mse_grad(capi.i64(n), capi.vp(y), capi.vp(t), capi.vp(gy), capi.vp(loss), None), "mse")
    d = (y.float() - t.float())
    assert abs(loss.item() - float((d * d).mean())) < 1e-4 * float((d * d).mean())
    assert torch.allclose(gy.float(), (2 * d / n).to(torch.bfloat16).float(), rtol=1e-2, atol=1e-6)
    w = torch.randn(50, device=cuda)
    g = torch.randn(50, device=cuda)
    m = torch.zeros(50, device=cuda)
    v = torch.zeros(50, device=cuda)
    wb = torch.zeros(50, dtype=torch.bfloat16, device=cuda)
    w0 = w.clone()
    capi.check(lib.sfem_gb300_adam_step(50, capi.vp(w), capi.vp(g), capi.vp(m), capi.vp(v), capi.vp(wb),
                                        ctypes.c_float(1e-2), ctypes.c_float(0.9), ctypes.c_float(0.999),
                                        ctypes.c_float(1e-8), 1, None), "adam")
    # first Adam step moves every weight by lr * sign(g)
    assert torch.allclose(w, w0 - 1e-2 * torch.sign(g), atol=1e-6)
    assert torch.allclose(wb.float(), w, rtol=1e-2, atol=1e-2)


@pytest.mark.parametrize("scaled", [True, False], ids=["inv_diag", "no_inv_diag"])
@pytest.mark.parametrize("shape", [(5, 4, 3), (1, 1, 1), (3, 3, 3)], ids=["60patches", "1patch", "27patches"])
@pytest.mark.parametrize("variant", [0, 1], ids=["tcgen05", "mma_sync"])
@pytest.mark.parametrize("dtype_name", ["float32", "float64"])
def test_fused_tensor_core_correction_matches_layer_kernels(cuda, dtype_name, variant, shape, scaled):
    """The fused tensor-core inference kernels (tcgen05 with tensor-memory accumulators, and
    warp-level mma.sync) against gather + three layer kernels + scatter (which the oracle
    pins): same network, same BF16 rounding points, FP32 accumulation in a different order,
    so agreement to BF16 resolution."""
    import torch

    from sfem_gb300.learned import PatchNet
    from sfem_gb300.mesh import SSMesh
    from sfem_gb300.solvers import Hierarchy

    dt = getattr(torch, dtype_name)
    m = SSMesh(*shape, 4, perturb=0.1, seed=1)
    H = Hierarchy(m, dirichlet_faces=("x0",), device=cuda)
    fine = H.spaces[0]
    P, N = m.n_elements, m.n_nodes()
    net = PatchNet(cuda, seed=3)
    for w in net.w32:  # larger output weights than the training init so the output is not tiny
        w.mul_(3.0)
    net.wbf = [w.to(torch.bfloat16) for w in net.w32]
    g = torch.Generator(device=cuda).manual_seed(5)
    r = torch.randn(N, dtype=dt, device=cuda, generator=g)
    inv = (torch.rand(N, dtype=dt, device=cuda, generator=g) + 0.5) if scaled else None
    lib = capi.load()
    frag = torch.empty(lib.sfem_gb300_learned_fragments_size(), dtype=torch.uint8, device=cuda)
    capi.check(lib.sfem_gb300_learned_fragments(capi.vp(net.wbf[0]), capi.vp(net.wbf[1]), capi.vp(net.wbf[2]),
                                                capi.vp(frag), None), "fragments")
    rt = capi.FLOAT32 if dt == torch.float32 else capi.FLOAT64
    d_fused = torch.zeros(N, dtype=dt, device=cuda)
    capi.check(lib.sfem_gb300_set_learned_kernel(variant), "variant")
    try:
        capi.check(lib.sfem_gb300_learned_correction(rt, capi.i64(P), fine.lidx_ptrs.ptr, capi.vp(r), capi.vp(inv),
                                                     capi.vp(frag), capi.vp(fine.count), ctypes.c_double(0.7),
                                                     capi.vp(d_fused), None), "fused")
        torch.cuda.synchronize()
    finally:
        capi.check(lib.sfem_gb300_set_learned_kernel(0), "variant")
    assert lib.sfem_gb300_learned_status() == 0
    a0 = torch.empty((P, 125), dtype=torch.bfloat16, device=cuda)
    ps = torch.empty(P, dtype=torch.float32, device=cuda)
    capi.check(lib.sfem_gb300_gather_patches(rt, capi.i64(P), fine.lidx_ptrs.ptr, capi.vp(r), capi.vp(inv),
                                             capi.vp(a0), capi.vp(ps), None), "gather")
    a1, a2, y = net.forward(a0)
    d_ref = torch.zeros(N, dtype=dt, device=cuda)
    capi.check(lib.sfem_gb300_scatter_patches(rt, capi.i64(P), fine.lidx_ptrs.ptr, capi.vp(y), capi.vp(ps),
                                              capi.vp(fine.count), ctypes.c_double(0.7), capi.vp(d_ref), None),
               "scatter")
    torch.cuda.synchronize()
    ref, got = d_ref.double(), d_fused.double()
    assert float(ref.abs().max()) > 0
    rel = float(torch.linalg.vector_norm(got - ref) / torch.linalg.vector_norm(ref))
    assert rel < 2e-2, rel
    assert float((got - ref).abs().max()) < 0.1 * float(ref.abs().max())


def test_learned_smoother_pipeline_small(cuda):
    """Harvest -> train (own BF16 kernels) -> FCG with the learned correction on a fresh
    coefficient draw: the loss drops and the solve reaches 1e-10 true residual."""
    from sfem_gb300 import learned

    res = learned.run_experiment(nx=8, draws=4, n_pairs=8000, epochs=8, eval_draws=1, device=str(cuda),
                                 placement="before")
    assert res["loss_last"] < res["loss_first"]
    row = res["eval"][0]
    for name in ("chebyshev3", "learned"):
        assert row[name]["rc"] == 0 and row[name]["true_rel_residual"] < 1e-10, row


def test_learned_smoother_gains_iterations(cuda):
    """What the trained network buys: on fresh coefficient draws of a 16^3 L=4 problem
    with k = exp(g) (sigma 1, correlation length 4 macro elements), FCG with the learned
    correction needs strictly fewer iterations than the same multigrid without it, both
    in FP64 and through the FP32 precision bridge, and every arm reaches 1e-10."""
    from sfem_gb300 import learned

    res = learned.run_experiment(nx=16, draws=16, n_pairs=30000, epochs=12, eval_draws=2, device=str(cuda),
                                 placement="before", fallback_sweeps=1)
    assert res["loss_last"] < 0.8 * res["loss_first"]
    for row in res["eval"]:
        for name in ("chebyshev3", "learned", "mixed", "mixed_learned"):
            assert row[name]["rc"] == 0 and row[name]["true_rel_residual"] < 1e-10, (name, row)
        assert row["learned"]["iterations"] < row["chebyshev3"]["iterations"], row
        assert row["mixed_learned"]["iterations"] < row["mixed"]["iterations"], row


def test_fallback_switch_recaptures_graph(cuda):
    """Graph-replayed V-cycles with the learned smoother: switching it to its Chebyshev3
    fallback must change what the replay runs (the graph is re-captured), so the switched
    solver takes exactly the plain V(2,2) multigrid's iterations and reaches its solution."""
    import torch

    from sfem_gb300 import learned
    from sfem_gb300 import solvers as S
    from sfem_gb300.mesh import SSMesh

    m = SSMesh(8, 8, 8, 4, perturb=0.1, seed=3)
    H = S.Hierarchy(m, dirichlet_faces=("x0",), device=cuda)
    g = torch.Generator(device=cuda).manual_seed(2)
    b = torch.randn(H.spaces[0].n_nodes, dtype=torch.float64, device=cuda, generator=g)
    b[H.dirichlet[0].long()] = 0
    net = learned.PatchNet(cuda, seed=1)

    def run(mg, op):
        solver = S.cg(S.context(), op, mg, rtol=1e-10, max_it=200, residual_norm=True, flexible=True)
        x = torch.zeros_like(b)
        assert S.solve(solver, b, x) == 0
        return S.stats(solver)[0], x

    ctx = S.context()
    mg_plain, op = S.build_poisson_mg(ctx, H, torch.float64, smoother="chebyshev3", sweeps=2, coarse="dense",
                                      graph=True)
    it_plain, x_plain = run(mg_plain, op)
    mg, op2 = learned.learned_mg(ctx, H, net, torch.float64, chain="before", coarse="dense", graph=True)
    it_learned, _ = run(mg, op2)  # captures the learned V-cycle
    learned.use_fallback(mg, True)
    it_fb, x_fb = run(mg, op2)
    assert it_fb == it_plain, (it_plain, it_learned, it_fb)
    assert float(torch.linalg.vector_norm(x_fb - x_plain) / torch.linalg.vector_norm(x_plain)) < 1e-8
