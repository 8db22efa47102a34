"""Batched serving: many independent sshex8 Poisson / elasticity solves at once.

No reference counterpart (the reference runs one solve per process,
``drivers/mgsolve.cpp``).  Problems are grouped by (kind, level L); within a
group the meshes of all problems are concatenated with node offsets, so every
element operator and transfer of the group is ONE launch of the single-problem
kernels over all its problems.  Vectors of all groups are concatenated again
into one batch vector (problem p owns a contiguous dof range), on which the
batched kernels of ``csrc/batched.cu`` run the per-problem Krylov algebra:

    FP64 flexible CG over the batch (per-problem scalars and masks, stop on
    ||r_p|| <= rtol ||b_p||), preconditioned through a per-problem precision bridge
      -> block-diagonal FP32 preconditioner: one multigrid V(s, s) per group
         (sshex8 levels, then hex8 levels coarsening each macro grid) with
         per-problem Chebyshev3 bounds and a batched Jacobi-PCG coarse solve.

Chunks of CG iterations are captured into a CUDA graph and replayed; the
autotuner picks the work-list chunk and CTA shape of the batched vector kernels
by timing the captured chunk.
"""

from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import capi
from . import solvers as S
from .mesh import CoarseHex8Level, SSMesh, derefinement_levels, perturbed_macro_points
from .operators import Laplacian

c_double = C.c_double
c_int = C.c_int


@dataclass(frozen=True)
class ProblemSpec:
    kind: str  # "poisson" | "elasticity"
    n: int  # macro elements per cube edge
    level: int  # micro level L
    seed: int

    @property
    def vec(self) -> int:
        return 3 if self.kind == "elasticity" else 1


def draw_problems(count=256, n_range=(8, 32), levels=(2, 3, 4), seed=0, kinds=("poisson", "elasticity")):
    """Seeded problem mix: kind uniform over ``kinds``, edge n uniform in n_range
    (inclusive), level uniform over ``levels``."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        kind = kinds[int(rng.integers(len(kinds)))]
        n = int(rng.integers(n_range[0], n_range[1] + 1))
        L = int(levels[int(rng.integers(len(levels)))])
        out.append(ProblemSpec(kind, n, L, int(seed * 100003 + i)))
    return out


_MESHES: dict = {}


def _mesh(n, L) -> SSMesh:
    """Numbering / connectivity of an n^3 cube at level L (geometry is per problem)."""
    key = (n, L)
    if key not in _MESHES:
        _MESHES[key] = SSMesh(n, n, n, L)
    return _MESHES[key]


def coarse_depth(n: int, min_nodes: int = 27) -> int:
    """Number of 2x coarsenings of an n^3 macro grid (odd edges keep a thin last
    element) while an edge has >= 2 elements and the next grid >= min_nodes nodes."""
    d = 0
    while n >= 2 and ((n + 1) // 2 + 1) ** 3 >= min_nodes:
        n = (n + 1) // 2
        d += 1
    return d


class _LevelSpace:
    """One level of a group: concatenated connectivity of its problems on the device."""

    def __init__(self, device, level, element_type, elements, n_nodes, n_elements, lidx=None, count=None, P=None,
                 R=None):
        import torch

        t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(device)
        self.level = level
        self.element_type = element_type
        self.n_nodes = n_nodes
        self.n_elements = n_elements
        self.device = device
        self.elements = t(elements)
        self.elements_ptrs = capi.DevicePtrArray(self.elements)
        self.is_macro_coarse = P is not None
        if lidx is not None:
            self.lidx_elements = t(lidx)
            self.lidx_ptrs = capi.DevicePtrArray(self.lidx_elements)
            self.count = t(count.view(np.int16))
        if self.is_macro_coarse:
            self.P = tuple(t(a) for a in P)
            self.R = tuple(t(a) for a in R)


def _block_diag_csr(blocks, row_offs, col_offs):
    """Concatenate per-problem CSR triples block-diagonally."""
    ptr, idx, val = [np.zeros(1, dtype=np.int64)], [], []
    nnz = 0
    for (rp, ci, w), co in zip(blocks, col_offs):
        ptr.append(rp[1:].astype(np.int64) + nnz)
        idx.append(ci.astype(np.int64) + co)
        val.append(w)
        nnz += int(rp[-1])
    return (np.concatenate(ptr).astype(np.int32), np.concatenate(idx).astype(np.int32), np.concatenate(val))


class BatchGroup:
    """All problems of one (kind, level, coarse depth): concatenated hierarchy, geometry, rhs.
    Transfers of the hex8 levels below the macro grids are block-diagonal CSR
    interpolations (one block per problem)."""

    def __init__(self, kind, level, problems, device, perturb=0.1, dirichlet_face="x0", depth=0):
        import torch

        self.kind, self.L, self.problems = kind, level, list(problems)
        self.vec = 3 if kind == "elasticity" else 1
        self.device = torch.device(device)
        self.levels = derefinement_levels(level)
        meshes = [_mesh(p.n, level) for p in self.problems]
        self.spaces, self.dirichlet, self.node_offsets = [], [], []
        for l in self.levels:
            offs = np.cumsum([0] + [m.n_nodes(l) for m in meshes])
            self.node_offsets.append(offs)
            els, lids, cnts, dns = [], [], [], []
            for m, o in zip(meshes, offs[:-1]):
                lid = m.elements(l)
                lids.append(lid + o)
                els.append((m.hex8_elements() if l == 1 else lid) + o)
                cnts.append(np.bincount(lid.reshape(-1), minlength=m.n_nodes(l)).astype(np.uint16))
                dns.append(m.boundary_nodes(dirichlet_face, l) + o)
            E = sum(m.n_elements for m in meshes)
            et = capi.HEX8 if l == 1 else capi.SSHEX8(l)
            self.spaces.append(_LevelSpace(self.device, l, et, np.concatenate(els, axis=1).astype(np.int32),
                                           int(offs[-1]), E, lidx=np.concatenate(lids, axis=1).astype(np.int32),
                                           count=np.concatenate(cnts)))
            self.dirichlet.append(torch.from_numpy(np.concatenate(dns).astype(np.int32)).to(self.device))
        self.n_sshex8 = len(self.spaces)
        # per-problem macro grids and their coarse hex8 chains
        grids = []
        for p, m in zip(self.problems, meshes):
            macro = perturbed_macro_points(p.n, p.n, p.n, perturb=perturb, seed=p.seed).astype(np.float32)
            K, J, I = np.meshgrid(np.arange(p.n + 1), np.arange(p.n + 1), np.arange(p.n + 1), indexing="ij")
            grids.append((macro, m.node_id(I * m.L, J * m.L, K * m.L)))
        chains = []
        for macro, ids in grids:
            chain = []
            for _ in range(depth):
                chain.append(CoarseHex8Level(macro, ids) if not chain else chain[-1].coarser())
            chains.append(chain)
        for c in range(depth):
            lv = [ch[c] for ch in chains]
            offs = np.cumsum([0] + [x.n_nodes for x in lv])
            fine_offs = self.node_offsets[-1]
            els = np.concatenate([x.hex8 + o for x, o in zip(lv, offs[:-1])], axis=1).astype(np.int32)
            P = _block_diag_csr([x.P for x in lv], fine_offs[:-1], offs[:-1])
            R = _block_diag_csr([x.R for x in lv], offs[:-1], fine_offs[:-1])
            sp = _LevelSpace(self.device, 1, capi.HEX8, els, int(offs[-1]), els.shape[1], P=P, R=R)
            sp.points_host = np.concatenate([x.points for x in lv], axis=1)
            self.spaces.append(sp)
            self.dirichlet.append(torch.from_numpy(np.concatenate(
                [x.boundary_nodes(dirichlet_face) + o for x, o in zip(lv, offs[:-1])]).astype(np.int32)).to(self.device))
            self.node_offsets.append(offs)
        self.n_nodes = int(self.node_offsets[0][-1])
        self.n_dofs = self.vec * self.n_nodes
        self._geometry(meshes, grids)

    def _fill(self, corners, points):
        import torch

        dev = self.device
        pts = torch.from_numpy(np.ascontiguousarray(points)).to(dev)
        cor = torch.from_numpy(np.ascontiguousarray(corners)).to(dev)
        pp, cp = capi.DevicePtrArray(pts), capi.DevicePtrArray(cor)
        E = cor.shape[1]
        lib = capi.load()
        fff = torch.empty((6, E), dtype=torch.float32, device=dev)
        capi.check(lib.sfem_gb300_hex8_fff_fill(capi.i64(E), cp.ptr, pp.ptr, capi.i64(E), capi.vp(fff), None),
                   "fff_fill")
        adj = torch.empty((9, E), dtype=torch.float32, device=dev)
        det = torch.empty(E, dtype=torch.float32, device=dev)
        capi.check(lib.sfem_gb300_hex8_adjugate_fill(capi.i64(E), cp.ptr, pp.ptr, capi.i64(E), capi.vp(adj),
                                                     capi.vp(det), None), "adjugate_fill")
        torch.cuda.synchronize(dev)
        return fff, adj, det

    def _geometry(self, meshes, grids):
        """Per-problem perturbed macro grids -> FFF / adjugate of every level."""
        pts, corners = [], []
        off = 0
        for (macro, ids), m in zip(grids, meshes):
            P1 = np.empty((3, m.n_nodes(1)), dtype=np.float32)
            P1[:, ids.reshape(-1)] = macro.reshape(3, -1)
            pts.append(P1)
            corners.append(m.hex8_elements() + off)
            off += m.n_nodes(1)
        fff, adj, det = self._fill(np.concatenate(corners, axis=1), np.concatenate(pts, axis=1))
        self.fff, self.adj, self.det = fff, adj, det
        for sp in self.spaces[:self.n_sshex8]:
            sp.fff, sp.adj, sp.det = fff, adj, det
        for sp in self.spaces[self.n_sshex8:]:
            sp.fff, sp.adj, sp.det = self._fill(sp.elements.cpu().numpy(), sp.points_host)

    def problem_dof_offsets(self, k=0):
        return self.vec * self.node_offsets[k]

    def rhs(self):
        """N(0,1) per dof (seeded per problem), zero on Dirichlet dofs."""
        parts = []
        for p, o0, o1 in zip(self.problems, self.node_offsets[0][:-1], self.node_offsets[0][1:]):
            parts.append(np.random.default_rng(p.seed + 7).standard_normal(self.vec * int(o1 - o0)))
        b = np.concatenate(parts)
        dn = self.dirichlet[0].cpu().numpy().astype(np.int64)
        for c in range(self.vec):
            b[self.vec * dn + c] = 0
        return b

    # ------------------------------------------------------------------ operators
    def op(self, ctx, k, dtype, tensor_cores=False):
        sp = self.spaces[k]
        if self.kind == "poisson":
            return S.laplacian_op(ctx, sp, sp.fff, self.dirichlet[k], dtype)
        return S.elasticity_op(ctx, sp, sp.adj, sp.det, 1.0, 10.0, self.dirichlet[k], dtype,
                               tensor_cores=tensor_cores)

    def diag(self, k, dtype):
        import torch

        sp = self.spaces[k]
        d = torch.zeros(self.vec * sp.n_nodes, dtype=dtype, device=self.device)
        if self.kind == "poisson":
            Laplacian(sp, packed=False).set_fff(sp.fff).hessian_diag(d)
        else:
            E = sp.n_elements
            capi.check(capi.load().sfem_gb300_linear_elasticity_block_diag(
                sp.element_type, capi.i64(E), sp.elements_ptrs.ptr, capi.i64(E), capi.vp(sp.adj),
                capi.vp(sp.det), c_double(1.0), c_double(10.0), S.rt_of(dtype), capi.vp(d), None, None), "diag")
        dn = self.dirichlet[k].long()
        for c in range(self.vec):
            d[self.vec * dn + c] = 1
        return d

    def transfer(self, ctx, k, dtype):
        C_, F = self.spaces[k + 1], self.spaces[k]
        if C_.is_macro_coarse:
            P = S.crs_transfer_op(ctx, C_.P, F.n_nodes, C_.n_nodes, self.vec, self.dirichlet[k], dtype)
            R = S.crs_transfer_op(ctx, C_.R, C_.n_nodes, F.n_nodes, self.vec, self.dirichlet[k + 1], dtype)
            return P, R
        P = S.prolongation_op(ctx, C_, F, self.vec, self.dirichlet[k], dtype)
        R = S.restriction_op(ctx, F, C_, self.vec, self.dirichlet[k + 1], dtype)
        return P, R


def _layout(ctx, dof_offsets, chunk=4096) -> S.Handle:
    offs = np.ascontiguousarray(np.asarray(dof_offsets, dtype=np.int64))
    return S._create(capi.load().sfem_gb300_batch_layout_create, ctx.ptr, c_int(len(offs) - 1),
                     offs.ctypes.data_as(C.c_void_p), c_int(chunk), keep=(ctx,))


class BatchSolver:
    """Mixed-precision batched solver over a list of :class:`ProblemSpec`."""

    def __init__(self, problems, device="cuda:0", sweeps=2, coarse_iterations=20, rtol=1e-10, max_it=300,
                 check_every=5, tensor_cores=False, use_graph=True, eigen_max_it=40, perturb=0.1,
                 coarse_min_nodes=27):
        import torch

        self.device = torch.device(device)
        self.ctx = S.context()
        ctx = self.ctx
        lib = capi.load()
        keyf = lambda p: (p.kind, p.level, coarse_depth(p.n, coarse_min_nodes))
        keys = sorted({keyf(p) for p in problems})
        self.groups = [BatchGroup(kd, L, [p for p in problems if keyf(p) == (kd, L, dp)], self.device,
                                  perturb=perturb, depth=dp) for kd, L, dp in keys]
        self.problems = [p for g in self.groups for p in g.problems]  # batch order
        self.layouts = []
        ops64, ops32, mgs, goffs = [], [], [], [0]
        for g in self.groups:
            nlev = len(g.spaces)
            mg = S.multigrid(ctx, torch.float32)
            for k in range(nlev):
                lay = _layout(ctx, g.problem_dof_offsets(k))
                self.layouts.append(lay)
                op = g.op(ctx, k, torch.float32)
                d = g.diag(k, torch.float32)
                if k == nlev - 1:
                    jac = S.jacobi(ctx, d, 1.0)
                    sm = S._create(lib.sfem_gb300_batch_cg_create, ctx.ptr, lay.ptr, op.ptr, jac.ptr,
                                   c_int(coarse_iterations), c_double(1e-6), c_int(0), keep=(ctx, lay, op, jac))
                else:
                    sop = g.op(ctx, k, torch.float32, tensor_cores=tensor_cores and g.kind == "elasticity")
                    inv = (1.0 / d).contiguous()
                    sm = S._create(lib.sfem_gb300_batch_chebyshev3_create, ctx.ptr, lay.ptr, sop.ptr, capi.vp(inv),
                                   c_int(sweeps), c_double(1.1 if g.kind == "elasticity" else 1.05), c_double(0.06),
                                   c_int(eigen_max_it), C.c_ulonglong(S.RANDOM_SEED), keep=(ctx, lay, sop, inv))
                P, R = g.transfer(ctx, k, torch.float32) if k + 1 < nlev else (None, None)
                S.mg_add_level(mg, op, sm, P, R)
            mgs.append(mg)
            ops32.append(g.op(ctx, 0, torch.float32))
            ops64.append(g.op(ctx, 0, torch.float64))
            goffs.append(goffs[-1] + g.n_dofs)
        self.group_offsets = np.asarray(goffs, dtype=np.int64)
        self.n = int(goffs[-1])
        dof_offs = [0]
        for g in self.groups:
            o = g.problem_dof_offsets(0)
            dof_offs += list(dof_offs[-1] + o[1:])
        self.dof_offsets = np.asarray(dof_offs, dtype=np.int64)
        self.layout = _layout(ctx, self.dof_offsets)
        self.layouts.append(self.layout)
        self.op64 = self._grouped(torch.float64, ops64)
        self.precond32 = self._grouped(torch.float32, mgs)
        self.bridge = S._create(lib.sfem_gb300_batch_bridge_create, ctx.ptr, self.layout.ptr, self.precond32.ptr,
                                keep=(ctx, self.layout, self.precond32))
        self.cg = S._create(lib.sfem_gb300_batch_cg_create, ctx.ptr, self.layout.ptr, self.op64.ptr, self.bridge.ptr,
                            c_int(1), c_double(rtol), c_int(1), keep=(ctx, self.layout, self.op64, self.bridge))
        self.solver = S._create(lib.sfem_gb300_batch_solve_create, ctx.ptr, self.layout.ptr, self.cg.ptr,
                                c_int(check_every), c_int(max_it), c_int(int(use_graph)), keep=(ctx, self.layout, self.cg))
        self.check_every = check_every
        self.tuned = None

    def _grouped(self, dtype, ops):
        arr = (C.c_void_p * len(ops))(*[o.ptr.value for o in ops])
        offs = np.ascontiguousarray(self.group_offsets)
        return S._create(capi.load().sfem_gb300_batch_grouped_op_create, self.ctx.ptr, c_int(S.rt_of(dtype)),
                         c_int(len(ops)), arr, offs.ctypes.data_as(C.c_void_p), keep=(self.ctx, *ops))

    @property
    def n_problems(self):
        return len(self.problems)

    def rhs(self):
        import torch

        return torch.from_numpy(np.concatenate([g.rhs() for g in self.groups])).to(self.device)

    def set_launch(self, chunk, threads, ctas_per_sm):
        for lay in self.layouts:
            capi.check(capi.load().sfem_gb300_batch_layout_set_launch(lay.ptr, c_int(chunk), c_int(threads),
                                                                       c_int(ctas_per_sm)), "set_launch")
        capi.check(capi.load().sfem_gb300_batch_solve_set_launch(self.solver.ptr, c_int(self.check_every)),
                   "solve_set_launch")

    def time_chunk(self, b, x, reps=1) -> float:
        ms = c_double(0)
        capi.check(capi.load().sfem_gb300_batch_solve_time_chunk(self.solver.ptr, capi.vp(b), capi.vp(x), c_int(reps),
                                                                 C.byref(ms)), "batch_solve_time_chunk")
        return ms.value

    # element-kernel tile shapes the autotuner tries: the FP32 sshex8 Laplacian
    # (sfem_gb300_set_laplacian_kernel: -1 per-level default, 0 staged tiles of 64
    # elements with one thread each, 2 one thread per element, 8 node-centric stencil
    # tiles of 32 elements x 4 warps) and the FP32 elasticity kernel
    # (sfem_gb300_set_elasticity_kernel: -1 default = tcgen05 pairs at L = 4, 0 SIMT warp
    # per element)
    KERNEL_CANDIDATES = {"laplacian": (-1, 0, 2, 8), "elasticity": (-1, 0)}

    def _set_kernels(self, kernels):
        """Select the element kernels; returns the previous selection."""
        lib = capi.load()
        prev = {"laplacian": lib.sfem_gb300_set_laplacian_kernel(int(kernels["laplacian"]))}
        old_e = getattr(self, "_elasticity_kernel", -1)
        capi.check(lib.sfem_gb300_set_elasticity_kernel(int(kernels["elasticity"])), "set_elasticity_kernel")
        self._elasticity_kernel = int(kernels["elasticity"])
        prev["elasticity"] = old_e
        return prev

    def autotune(self, b, candidates=None, reps=1, kernels=None):
        """Pick the element kernels (tile shapes) of the group operators and the launch
        shape (chunk, threads per CTA, CTAs per SM) of the batched vector kernels by
        timing a captured chunk of CG iterations on a scratch iterate: first each
        operator family's kernel candidates at the first launch shape, then the launch
        shapes with the chosen kernels.  Returns the timing table."""
        import torch

        if candidates is None:
            candidates = [(2048, 256, 8), (4096, 256, 8), (8192, 512, 4), (4096, 128, 16)]
        if kernels is None:
            kernels = self.KERNEL_CANDIDATES
        table = []
        best = {"laplacian": -1, "elasticity": -1}
        self.set_launch(*candidates[0])
        saved = None
        try:
            for family, kind in (("laplacian", "poisson"), ("elasticity", "elasticity")):
                if not any(g.kind == kind for g in self.groups) or len(kernels[family]) < 2:
                    continue
                timed = []
                for v in kernels[family]:
                    prev = self._set_kernels({**best, family: v})
                    saved = saved or prev
                    xs = torch.zeros_like(b)
                    t = self.time_chunk(b, xs, reps)
                    timed.append((t, v))
                    table.append((candidates[0], {**best, family: v}, t))
                best[family] = min(timed)[1]
            prev = self._set_kernels(best)
            saved = saved or prev
            for cand in candidates:
                self.set_launch(*cand)
                xs = torch.zeros_like(b)
                table.append((cand, dict(best), self.time_chunk(b, xs, reps)))
        finally:
            if saved is not None:
                self._set_kernels(saved)
        launch_rows = [t for t in table if t[1] == best]
        best_launch = min(launch_rows, key=lambda t: t[2])[0]
        self.set_launch(*best_launch)
        self.tuned = best_launch
        self.tuned_kernels = dict(best)
        return table

    def solve(self, b, x, release=None):
        """Solve every problem to ||b_p - A_p x_p|| <= rtol ||b_p|| (FP64, zero start).
        ``release`` (seconds from the start of the call, one per problem in batch order)
        staggers the arrivals: a problem iterates from the first chunk boundary after its
        release.  Returns (rc, per-problem latency s from release, per-problem
        iterations, seconds)."""
        P = self.n_problems
        lat = np.zeros(P)
        its = np.zeros(P, dtype=np.int32)
        sec = c_double(0)
        lib = capi.load()
        prev = self._set_kernels(self.tuned_kernels) if getattr(self, "tuned_kernels", None) else None
        try:
            rc = self._run(lib, b, x, release, P, lat, its, sec)
        finally:
            if prev is not None:
                self._set_kernels(prev)
        return rc, lat, its, sec.value

    def _run(self, lib, b, x, release, P, lat, its, sec):
        if release is None:
            rc = lib.sfem_gb300_batch_solve_run(self.solver.ptr, capi.vp(b), capi.vp(x), lat.ctypes.data_as(C.c_void_p),
                                                its.ctypes.data_as(C.c_void_p), C.byref(sec))
        else:
            rel = np.ascontiguousarray(release, dtype=np.float64)
            if rel.shape != (P,):
                raise ValueError(f"release: {P} times expected, got shape {rel.shape}")
            rc = lib.sfem_gb300_batch_solve_run_released(self.solver.ptr, capi.vp(b), capi.vp(x),
                                                         rel.ctypes.data_as(C.c_void_p), lat.ctypes.data_as(C.c_void_p),
                                                         its.ctypes.data_as(C.c_void_p), C.byref(sec))
        return rc

    def true_residuals(self, b, x):
        """||b_p - A_p x_p|| / ||b_p|| per problem with the FP64 operators (device)."""
        import torch

        r = torch.zeros_like(b)
        S.apply(self.op64, x, r)
        r = b - r
        rr = torch.zeros(self.n_problems, dtype=torch.float64, device=self.device)
        bb = torch.zeros_like(rr)
        lib = capi.load()
        capi.check(lib.sfem_gb300_batch_dot(self.layout.ptr, capi.FLOAT64, capi.vp(r), capi.vp(r), capi.vp(rr)), "dot")
        capi.check(lib.sfem_gb300_batch_dot(self.layout.ptr, capi.FLOAT64, capi.vp(b), capi.vp(b), capi.vp(bb)), "dot")
        return (rr.sqrt() / bb.sqrt()).cpu().numpy()


def stream_priority_levels(sizes, levels=6):
    """Stream priority level per group (0 = the default, higher = scheduled first): the
    groups ranked by size, the smallest on the top level (levels - 1), the largest on 0,
    the ranks in between spread over the levels (equal sizes keep their order).  One
    group: level 0."""
    n = len(sizes)
    out = [0] * n
    if n < 2:
        return out
    order = sorted(range(n), key=lambda i: sizes[i])
    for rank, i in enumerate(order):
        out[i] = (levels - 1) - (rank * (levels - 1)) // (n - 1)
    return out


class ConcurrentBatchSolver:
    """The problems of a :class:`BatchSolver`, one batched solver per group (its own
    context, stream and captured chunk of CG iterations), advanced independently by one
    host loop: a group launches its next chunk as soon as the convergence mask of its
    last chunk has arrived (``sfem_gb300_batch_solve_begin / step / poll``).  Kernels of
    different groups overlap on the GPU, and a group of small problems finishes on its
    own cadence instead of the slowest group's."""

    PRIORITY_LEVELS = 6  # stream priority steps used (clamped to the device's range)

    def __init__(self, problems, device="cuda:0", launch=None, kernels=None, coarse_min_nodes=27, prioritize=True,
                 **kw):
        keyf = lambda p: (p.kind, p.level, coarse_depth(p.n, coarse_min_nodes))
        keys = sorted({keyf(p) for p in problems})
        self.subs = [BatchSolver([p for p in problems if keyf(p) == k], device=device,
                                 coarse_min_nodes=coarse_min_nodes, **kw) for k in keys]
        if launch is not None:
            for s in self.subs:
                s.set_launch(*launch)
        # the smaller a group's total dofs, the higher its stream priority: its chunks
        # are short, and running them first is what takes its problems out of the queue
        self.priority = (stream_priority_levels([g.n for g in self.subs], self.PRIORITY_LEVELS) if prioritize
                         else [0] * len(self.subs))
        for sub, level in zip(self.subs, self.priority):
            if level:
                capi.check(capi.load().sfem_gb300_batch_solve_set_priority(sub.solver.ptr, C.c_int(level)),
                           "batch_solve_set_priority")
        self.kernels = dict(kernels) if kernels else None
        self.problems = [p for s in self.subs for p in s.problems]
        self.offsets = np.cumsum([0] + [s.n_problems for s in self.subs])

    @property
    def n_problems(self):
        return len(self.problems)

    def rhs(self):
        """One right-hand side per group (in group order)."""
        return [s.rhs() for s in self.subs]

    def solve(self, bs, xs):
        """Solve every group's problems to ||b_p - A_p x_p|| <= rtol ||b_p|| (zero start),
        all submitted at once.  Returns (per-problem latency s, per-problem iterations,
        seconds); a problem's latency is when the host saw its group's mask drop it."""
        import time

        lib = capi.load()
        P = self.n_problems
        lat = np.zeros(P)
        its = np.zeros(P, dtype=np.int32)
        n = len(self.subs)
        masks = [np.zeros(s.n_problems, dtype=np.int32) for s in self.subs]
        prev = [None] * n
        done = [False] * n
        saved = self.subs[0]._set_kernels(self.kernels) if self.kernels else None
        try:
            t0 = time.perf_counter()
            for s, b, x in zip(self.subs, bs, xs):
                capi.check(lib.sfem_gb300_batch_solve_begin(s.solver.ptr, capi.vp(b), capi.vp(x)), "batch_solve_begin")
            n_act, it = C.c_int(0), C.c_int(0)
            while not all(done):
                for i, s in enumerate(self.subs):
                    if done[i]:
                        continue
                    rc = lib.sfem_gb300_batch_solve_poll(s.solver.ptr, masks[i].ctypes.data_as(C.c_void_p),
                                                         C.byref(n_act), C.byref(it))
                    if rc == 2:  # this group's chunk is still running
                        continue
                    capi.check(rc, "batch_solve_poll")
                    now = time.perf_counter() - t0
                    if prev[i] is not None:
                        conv = (prev[i] != 0) & (masks[i] == 0)
                        lat[self.offsets[i]:self.offsets[i + 1]][conv] = now
                        its[self.offsets[i]:self.offsets[i + 1]][conv] = it.value
                    prev[i] = masks[i].copy()
                    if n_act.value == 0:
                        done[i] = True
                        continue
                    capi.check(lib.sfem_gb300_batch_solve_step(s.solver.ptr), "batch_solve_step")
            seconds = time.perf_counter() - t0
        finally:
            if saved is not None:
                self.subs[0]._set_kernels(saved)
        return lat, its, seconds

    def true_residuals(self, bs, xs):
        return np.concatenate([s.true_residuals(b, x) for s, b, x in zip(self.subs, bs, xs)])
