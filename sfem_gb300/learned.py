"""Learned multigrid smoother for sshex8 (L=4) Laplacians with heterogeneous coefficients.

No reference counterpart.  Pipeline (every numeric step runs in the CUDA
library through the C ABI; torch only holds device memory):

1. ``harvest``: for each coefficient draw, solve A x* = b with the plain
   (Chebyshev3) multigrid, then run plain V-cycles as a stationary iteration
   and record, after every coarse-grid correction of the finest level, the
   residual r = b - A x_cc and the error e = x* - x_cc.  Per macro element the
   5x5x5 patches of D^-1 r (input) and e (target) are normalised by the RMS of
   the input patch.
2. ``train``: Adam on the MSE between the network output and the target
   patches, with the hand-written BF16 forward / backward kernels.
3. ``learned_mg``: the same hierarchy with the finest-level smoother replaced
   by ``sweeps`` learned corrections (Chebyshev3 kept as fallback), used as
   the preconditioner of flexible CG.
"""

from __future__ import annotations

import ctypes as C
import time

import numpy as np

from . import capi
from . import solvers as S
from .mesh import coarsen_coefficient

CH = 16


def _lib():
    return capi.load()


class PatchNet:
    """3-layer 3x3x3 conv net 1 -> 16 -> 16 -> 1 (ReLU between layers), BF16 weights."""

    def __init__(self, device, seed=0, channels=CH):
        import torch

        self.device = device
        self.ch = channels
        g = np.random.default_rng(seed)
        shapes = [(channels, 1), (channels, channels), (1, channels)]
        self.shapes = shapes
        self.w32, self.wbf, self.m, self.v, self.g = [], [], [], [], []
        for co, ci in shapes:
            w = g.standard_normal(co * ci * 27) * np.sqrt(2.0 / (ci * 27))
            if co == 1:
                w *= 0.1  # small initial corrections
            t = torch.from_numpy(w.astype(np.float32)).to(device)
            self.w32.append(t)
            self.wbf.append(t.to(torch.bfloat16))
            self.m.append(torch.zeros_like(t))
            self.v.append(torch.zeros_like(t))
            self.g.append(torch.zeros_like(t))
        self.step = 0

    def state_dict(self):
        return {f"w{k}": w.cpu().numpy() for k, w in enumerate(self.w32)}

    def load_state_dict(self, d):
        import torch

        for k in range(3):
            self.w32[k].copy_(torch.from_numpy(d[f"w{k}"]))
            self.wbf[k].copy_(self.w32[k].to(torch.bfloat16))

    def forward(self, x):
        """x: [P, 125] BF16 -> activations (a1, a2, y)."""
        import torch

        P = x.shape[0]
        lib = _lib()
        a1 = torch.empty((P, 125, self.ch), dtype=torch.bfloat16, device=self.device)
        a2 = torch.empty_like(a1)
        y = torch.empty((P, 125), dtype=torch.bfloat16, device=self.device)
        capi.check(lib.sfem_gb300_patchconv_forward(capi.i64(P), 1, self.ch, capi.vp(x), capi.vp(self.wbf[0]), 1,
                                                    capi.vp(a1), None), "fwd1")
        capi.check(lib.sfem_gb300_patchconv_forward(capi.i64(P), self.ch, self.ch, capi.vp(a1), capi.vp(self.wbf[1]),
                                                    1, capi.vp(a2), None), "fwd2")
        capi.check(lib.sfem_gb300_patchconv_forward(capi.i64(P), self.ch, 1, capi.vp(a2), capi.vp(self.wbf[2]), 0,
                                                    capi.vp(y), None), "fwd3")
        return a1, a2, y

    def train_step(self, x, target, lr=1e-3):
        """One Adam step on a batch; returns the (pre-step) loss (device tensor)."""
        import torch

        P = x.shape[0]
        lib = _lib()
        a1, a2, y = self.forward(x)
        gy = torch.empty_like(y)
        loss = torch.zeros(1, dtype=torch.float32, device=self.device)
        capi.check(lib.sfem_gb300_mse_grad(capi.i64(P * 125), capi.vp(y), capi.vp(target), capi.vp(gy), capi.vp(loss),
                                           None), "mse")
        for gw in self.g:
            gw.zero_()
        g2 = torch.empty_like(a2)
        g1 = torch.empty_like(a1)
        # layer 3 (16 -> 1), input a2 went through ReLU
        capi.check(lib.sfem_gb300_patchconv_backward_weights(capi.i64(P), self.ch, 1, capi.vp(gy), capi.vp(a2),
                                                             capi.vp(self.g[2]), None), "bw3")
        capi.check(lib.sfem_gb300_patchconv_backward_data(capi.i64(P), self.ch, 1, capi.vp(gy), capi.vp(self.wbf[2]),
                                                          capi.vp(a2), capi.vp(g2), None), "bd3")
        capi.check(lib.sfem_gb300_patchconv_backward_weights(capi.i64(P), self.ch, self.ch, capi.vp(g2), capi.vp(a1),
                                                             capi.vp(self.g[1]), None), "bw2")
        capi.check(lib.sfem_gb300_patchconv_backward_data(capi.i64(P), self.ch, self.ch, capi.vp(g2),
                                                          capi.vp(self.wbf[1]), capi.vp(a1), capi.vp(g1), None), "bd2")
        capi.check(lib.sfem_gb300_patchconv_backward_weights(capi.i64(P), 1, self.ch, capi.vp(g1), capi.vp(x),
                                                             capi.vp(self.g[0]), None), "bw1")
        self.step += 1
        for k in range(3):
            capi.check(lib.sfem_gb300_adam_step(self.w32[k].numel(), capi.vp(self.w32[k]), capi.vp(self.g[k]),
                                                capi.vp(self.m[k]), capi.vp(self.v[k]), capi.vp(self.wbf[k]),
                                                C.c_float(lr), C.c_float(0.9), C.c_float(0.999), C.c_float(1e-8),
                                                self.step, None), "adam")
        return loss


def _gather(space_lidx_ptrs, P, v, scale, out, pscale, dtype):
    capi.check(_lib().sfem_gb300_gather_patches(S.rt_of(dtype), capi.i64(P), space_lidx_ptrs.ptr, capi.vp(v),
                                                capi.vp(scale), capi.vp(out), capi.vp(pscale), None), "gather")


def harvest(H, dtype, cycles=4, n_patches=None, seed=0, rhs=None, mg=None, ctx=None, point="cycle", target="local"):
    """(input, target) BF16 patch pairs from plain V-cycles on the hierarchy ``H``.

    point="cycle": pairs (D^-1 r_k, e_k) after every complete V-cycle of the stationary
    iteration x_{k+1} = x_k + MG(b - A x_k) (what a correction applied after the cycle's
    post-smoothing sees); point="coarse": after each coarse-grid correction of the finest
    level, before post-smoothing.

    target="local": the error patch minus its trilinear interpolant from the 8 macro
    corners, i.e. the part of the error the coarse levels cannot represent and the
    patch residual can predict; target="full": the error patch itself."""
    import torch

    ctx = ctx or S.context()
    fine = H.spaces[0]
    N = fine.n_nodes
    P = H.mesh.n_elements
    dev = H.device
    if mg is None:
        mg, _ = S.build_poisson_mg(ctx, H, dtype, smoother="chebyshev3", sweeps=2)
    op = S.laplacian_op(ctx, fine, H.fff, H.dirichlet[0], dtype)
    g = torch.Generator(device=dev).manual_seed(seed)
    b = rhs if rhs is not None else torch.randn(N, dtype=dtype, device=dev, generator=g)
    b[H.dirichlet[0].long()] = 0
    # exact solution of the fine system
    solver = S.cg(ctx, op, mg, rtol=1e-7 if dtype == torch.float32 else 1e-12, max_it=200, residual_norm=True,
                  flexible=True)
    xs = torch.zeros_like(b)
    S.solve(solver, b, xs)
    inv_diag = fine_inv_diag(H, dtype)
    xcc = torch.zeros_like(b)
    x = torch.zeros_like(b)
    if point == "coarse":
        capi.check(_lib().sfem_gb300_mg_set_harvest(mg.ptr, capi.vp(xcc)), "harvest")
    else:
        xcc = x
    ins, tgts = [], []
    pin = torch.empty((P, 125), dtype=torch.bfloat16, device=dev)
    ps = torch.empty(P, dtype=torch.float32, device=dev)
    tmp = torch.empty((P, 125), dtype=torch.bfloat16, device=dev)
    ones = torch.ones(P, dtype=torch.float32, device=dev)
    for c in range(cycles):
        S.solve(mg, b, x)  # one V-cycle in place (x is the running iterate)
        r = torch.zeros_like(b)
        S.apply(op, xcc, r)
        r = b - r
        e = xs - xcc
        _gather(fine.lidx_ptrs, P, r, inv_diag, pin, ps, dtype)
        # target: e patches scaled by the input patch's RMS
        _gather(fine.lidx_ptrs, P, e, None, tmp, torch.empty_like(ps), dtype)
        tscale = _patch_rms(e, fine, P, dtype)
        tgt = tmp.float() * (tscale / ps)[:, None]
        if target == "local":
            W, corners = _corner_interp(dev)
            tgt = tgt - tgt[:, corners] @ W.T
        tgt = tgt.to(torch.bfloat16)
        ins.append(pin.clone())
        tgts.append(tgt)
    if point == "coarse":
        capi.check(_lib().sfem_gb300_mg_set_harvest(mg.ptr, None), "harvest off")
    xin = torch.cat(ins)
    xt = torch.cat(tgts)
    if n_patches is not None and n_patches < xin.shape[0]:
        idx = torch.randperm(xin.shape[0], generator=torch.Generator(device=dev).manual_seed(seed + 1), device=dev)
        idx = idx[:n_patches]
        xin, xt = xin[idx], xt[idx]
    return xin, xt


def _corner_interp(device, L=4):
    """([125, 8] trilinear weights, the 8 corner positions) of an (L+1)^3 micro grid, lidx order."""
    import torch

    n1 = L + 1
    corners = [(cz * n1 + cy) * n1 + cx for cz in (0, L) for cy in (0, L) for cx in (0, L)]
    t = np.arange(n1) / L
    W = np.zeros((n1 ** 3, 8))
    for z in range(n1):
        for y in range(n1):
            for x in range(n1):
                k = 0
                for wz in (1 - t[z], t[z]):
                    for wy in (1 - t[y], t[y]):
                        for wx in (1 - t[x], t[x]):
                            W[(z * n1 + y) * n1 + x, k] = wz * wy * wx
                            k += 1
    return torch.from_numpy(W).float().to(device), torch.tensor(corners, device=device)


def _patch_rms(v, space, P, dtype):
    import torch

    out = torch.empty((P, 125), dtype=torch.bfloat16, device=v.device)
    s = torch.empty(P, dtype=torch.float32, device=v.device)
    _gather(space.lidx_ptrs, P, v, None, out, s, dtype)
    return s


def fine_inv_diag(H, dtype):
    import torch

    from .operators import Laplacian

    sp = H.spaces[0]
    d = torch.zeros(sp.n_nodes, dtype=dtype, device=H.device)
    Laplacian(sp, packed=False).set_fff(H.fff).hessian_diag(d)
    d[H.dirichlet[0].long()] = 1
    return 1.0 / d


def train(net: PatchNet, xin, xt, epochs=20, batch=4096, lr=2e-3, seed=0, log=None):
    import torch

    n = xin.shape[0]
    g = torch.Generator(device=xin.device).manual_seed(seed)
    history = []
    for ep in range(epochs):
        perm = torch.randperm(n, generator=g, device=xin.device)
        tot = torch.zeros(1, device=xin.device)
        nb = 0
        for s in range(0, n, batch):
            idx = perm[s:s + batch]
            tot += net.train_step(xin[idx].contiguous(), xt[idx].contiguous(), lr=lr)
            nb += 1
        history.append(float(tot.item()) / nb)
        if log:
            log(f"epoch {ep}: loss {history[-1]:.5f}")
    return history


def learned_mg(ctx, H, net: PatchNet, dtype, omega=1.0, sweeps=1, eig_max=None, post_only=False, chain=True,
               fallback_sweeps=None, **mg_kwargs):
    """Multigrid with the learned smoother on the finest level.

    chain="before" : the finest-level post-smoothing is the learned correction of the
    coarse-grid-corrected iterate followed by Chebyshev3 (matches point="coarse" data);
    chain=True (or "after"): Chebyshev3 followed by the learned correction (matches
    point="cycle" data); chain=False: the learned smoother replaces Chebyshev3 (pre and
    post unless post_only).  fallback_sweeps: Chebyshev3 sweeps of the post-smoother that
    follows (or precedes) the learned correction (default: the pre-smoother's 2)."""
    mg, op = S.build_poisson_mg(ctx, H, dtype, smoother="chebyshev3", sweeps=2, eig_max=eig_max, **mg_kwargs)
    fine = H.spaces[0]
    inv_diag = fine_inv_diag(H, dtype)
    lib = _lib()
    ch = mg.smoothers[0]  # finest-level Chebyshev3: the fallback
    if fallback_sweeps is not None and fallback_sweeps != 2:
        ch = S.chebyshev3(ctx, op, max_it=fallback_sweeps, eig_max=mg.eigs[0], inv_diag=inv_diag)
        mg.keep.append(ch)
    out = C.c_void_p(0)
    capi.check(lib.sfem_gb300_learned_smoother_create(
        ctx.ptr, op.ptr, fine.lidx_ptrs.ptr, capi.i64(H.mesh.n_elements), capi.vp(fine.count), capi.vp(inv_diag),
        capi.vp(net.wbf[0]), capi.vp(net.wbf[1]), capi.vp(net.wbf[2]), net.ch, C.c_double(omega), sweeps, ch.ptr,
        C.byref(out)), "learned smoother")
    ls = S.Handle(out, keep=(ctx, op, inv_diag, net, ch))
    if chain:
        capi.check(lib.sfem_gb300_learned_smoother_set_chain(ls.ptr, 2 if chain == "before" else 1), "chain")
        capi.check(lib.sfem_gb300_mg_set_post_smoother(mg.ptr, 0, ls.ptr), "post smoother")
    elif post_only:
        capi.check(lib.sfem_gb300_mg_set_post_smoother(mg.ptr, 0, ls.ptr), "post smoother")
    else:
        # replace both pre- and post-smoothing on the finest level
        capi.check(lib.sfem_gb300_mg_set_post_smoother(mg.ptr, 0, ls.ptr), "post smoother")
        capi.check(lib.sfem_gb300_mg_set_pre_smoother(mg.ptr, 0, ls.ptr), "pre smoother")
    mg.keep.append(ls)
    mg.learned = ls
    return mg, op


def use_fallback(mg, flag=True):
    capi.check(_lib().sfem_gb300_learned_smoother_use_fallback(mg.learned.ptr, int(flag)), "fallback")


def set_fallback(solver, mg):
    capi.check(_lib().sfem_gb300_solver_set_fallback(solver.ptr, mg.learned.ptr), "set_fallback")


def fallback_used(solver) -> bool:
    v = C.c_int(0)
    _lib().sfem_gb300_solver_fallback_used(solver.ptr, C.byref(v))
    return bool(v.value)


def hierarchy_with_coefficient(mesh, k, device, base=None, coarsen_macro=True):
    """Hierarchy of ``mesh`` whose metric is scaled per macro element by ``k`` (reuses
    ``base``'s device mesh).  The metrics are rescaled in place, so every level and
    every operator built on them sees the coefficient; hex8 levels below the macro
    mesh take the mean of their children's coefficients."""
    import torch

    if base is None:
        base = S.Hierarchy(mesh, dirichlet_faces=("x0",), device=device, coarsen_macro=coarsen_macro)
        base.fff_unscaled = [sp.fff.clone() for sp in base.spaces]
    kk = np.asarray(k, dtype=np.float64).reshape(mesh.nz, mesh.ny, mesh.nx)
    for i, sp in enumerate(base.spaces):
        if getattr(sp, "is_macro_coarse", False):
            cx, cy, cz = sp.lvl.shape
            kk = coarsen_coefficient(kk, (cz, cy, cx))
            kt = torch.as_tensor(kk.reshape(-1), dtype=torch.float32, device=base.device)
        else:
            kt = torch.as_tensor(np.asarray(k, dtype=np.float64), dtype=torch.float32, device=base.device)
        sp.fff.copy_(base.fff_unscaled[i] * kt[None, :])
    return base


def run_experiment(nx=32, draws=64, n_pairs=100_000, epochs=30, eval_draws=2, device="cuda:0", seed=0, log=None,
                   rtol=1e-10, placement="before", arms=("chebyshev3", "learned", "mixed", "mixed_learned"),
                   graph=True, fallback_sweeps=None):
    """Train on ``draws`` coefficient fields, then A/B on fresh draws: FP64 flexible CG
    preconditioned by the FP64 multigrid (chebyshev3), the same plus the learned correction
    (learned), the FP32 multigrid through the precision bridge (mixed), and that plus the
    learned correction (mixed_learned).

    placement="before": pairs harvested after each coarse-grid correction of the finest
    level and the correction applied there, before the Chebyshev3 post-smoothing;
    "after": pairs after complete V-cycles, correction after the post-smoothing.
    graph=True replays every arm's V-cycle as a captured CUDA graph (the learned
    correction has no host synchronisation; a switch to the fallback re-captures)."""
    import torch

    from .coefficients import lognormal_coefficient
    from .mesh import SSMesh

    dev = torch.device(device)
    mesh = SSMesh(nx, nx, nx, 4)
    H = None
    per_draw = max(1, n_pairs // draws)
    xs, ts = [], []
    t0 = time.perf_counter()
    ctx = S.context()
    for d in range(draws):
        k = lognormal_coefficient(nx, nx, nx, ell=8.0 * nx / 32.0, sigma=1.0, seed=seed + 1000 + d)
        H = hierarchy_with_coefficient(mesh, k, dev, H)
        xin, xt = harvest(H, torch.float32, cycles=3, n_patches=per_draw, seed=seed + d, ctx=ctx,
                          point="coarse" if placement == "before" else "cycle")
        xs.append(xin)
        ts.append(xt)
    xin, xt = torch.cat(xs), torch.cat(ts)
    t_harvest = time.perf_counter() - t0
    net = PatchNet(dev, seed=seed)
    t0 = time.perf_counter()
    hist = train(net, xin, xt, epochs=epochs, log=log)
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t0
    results = []
    chain = "before" if placement == "before" else True
    for d in range(eval_draws):
        k = lognormal_coefficient(nx, nx, nx, ell=8.0 * nx / 32.0, sigma=1.0, seed=seed + 5000 + d)
        H = hierarchy_with_coefficient(mesh, k, dev, H)
        g = torch.Generator(device=dev).manual_seed(seed + 77 + d)
        b = torch.randn(H.spaces[0].n_nodes, dtype=torch.float64, device=dev, generator=g)
        b[H.dirichlet[0].long()] = 0
        row = {}
        # FP64 flexible CG in every arm; the preconditioner differs: FP64 multigrid with or
        # without the learned correction, FP32 multigrid (bridged) with or without it
        for name in arms:
            ctx = S.context()
            learned_arm = name.endswith("learned")
            if name in ("chebyshev3", "learned"):
                mg, op = (learned_mg(ctx, H, net, torch.float64, chain=chain, coarse="dense", graph=graph,
                                     fallback_sweeps=fallback_sweeps)
                          if learned_arm else
                          S.build_poisson_mg(ctx, H, torch.float64, smoother="chebyshev3", sweeps=2, coarse="dense",
                                             graph=graph))
                pc, op64 = mg, op
            else:
                mg, _ = (learned_mg(ctx, H, net, torch.float32, chain=chain, coarse="dense", graph=graph,
                                    fallback_sweeps=fallback_sweeps)
                         if learned_arm else
                         S.build_poisson_mg(ctx, H, torch.float32, smoother="chebyshev3", sweeps=2, coarse="dense",
                                            graph=graph))
                op64 = S.laplacian_op(ctx, H.spaces[0], H.spaces[0].fff, H.dirichlet[0], torch.float64)
                pc = S.mixed_precond(ctx, mg)
            solver = S.cg(ctx, op64, pc, rtol=rtol, max_it=500, residual_norm=True, flexible=True)
            if learned_arm:
                set_fallback(solver, mg)
            x = torch.zeros_like(b)
            torch.cuda.synchronize()
            t1 = time.perf_counter()
            rc = S.solve(solver, b, x)
            torch.cuda.synchronize()
            dt = time.perf_counter() - t1
            r = torch.zeros_like(b)
            S.apply(op64, x, r)
            true_rel = float(torch.linalg.vector_norm(b - r) / torch.linalg.vector_norm(b))
            it, _ = S.stats(solver)
            row[name] = {"iterations": it, "seconds": dt, "true_rel_residual": true_rel, "rc": rc,
                         "fallback_used": fallback_used(solver) if learned_arm else False}
        results.append(row)
    return {"nx": nx, "draws": draws, "pairs": int(xin.shape[0]), "epochs": epochs, "placement": placement,
            "loss_first": hist[0],
            "loss_last": hist[-1], "harvest_seconds": t_harvest, "train_seconds": t_train, "eval": results,
            "net": net}
