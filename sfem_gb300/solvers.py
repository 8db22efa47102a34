"""Python binding of the device solver object layer (operators, smoothers, CG, multigrid).

Mirrors the reference's frontend composition of a geometric multigrid on a
semi-structured mesh (``create_gmg_data``, ``algebra/mg/sfem_GeometricMultigrid.cpp:12-167``;
``drivers/mgsolve.cpp:128-330``): one operator per derefinement level, nested
prolongation / restriction with Dirichlet zeroing, a smoother per level
(Chebyshev3 or Jacobi sweeps), a Jacobi-PCG coarse solve, and an outer CG
preconditioned by one V-cycle.  Every call goes through the C ABI of
``libsfem_gb300.so``; torch tensors only hold device memory.
"""

from __future__ import annotations

import ctypes as C

import numpy as np

from . import capi
from .mesh import CoarseHex8Level, SSMesh, coarsen_coefficient, macro_coarse_levels
from .operators import Laplacian, SSMeshDevice

c_double = C.c_double
c_int = C.c_int


def _lib():
    return capi.load()


class Handle:
    """Owns one opaque handle of the C ABI (released with sfem_gb300_handle_destroy)."""

    def __init__(self, ptr, keep=()):
        self.ptr = C.c_void_p(ptr.value if isinstance(ptr, C.c_void_p) else ptr)
        self.keep = list(keep)

    def __del__(self):
        try:
            if self.ptr and self.ptr.value:
                _lib().sfem_gb300_handle_destroy(self.ptr)
                self.ptr = C.c_void_p(0)
        except Exception:
            pass


def _create(fn, *args, keep=()):
    out = C.c_void_p(0)
    capi.check(fn(*args, C.byref(out)), fn.__name__)
    return Handle(out, keep)


def context(stream=None) -> Handle:
    return _create(_lib().sfem_gb300_context_create, stream)


def rt_of(dtype) -> int:
    import torch

    return capi.FLOAT32 if dtype == torch.float32 else capi.FLOAT64


def apply(op: Handle, x, y):
    capi.check(_lib().sfem_gb300_op_apply(op.ptr, capi.vp(x), capi.vp(y)), "sfem_gb300_op_apply")
    return y


def solve(solver: Handle, b, x):
    rc = _lib().sfem_gb300_solver_apply(solver.ptr, capi.vp(b), capi.vp(x))
    return rc


def stats(solver: Handle):
    it = c_int(0)
    rel = c_double(0)
    _lib().sfem_gb300_solver_stats(solver.ptr, C.byref(it), C.byref(rel))
    return it.value, rel.value


def laplacian_op(ctx, space: SSMeshDevice, fff, dirichlet, dtype) -> Handle:
    E = space.n_elements
    return _create(_lib().sfem_gb300_laplacian_op_create, ctx.ptr, c_int(rt_of(dtype)), c_int(space.element_type),
                   capi.i64(E), space.elements_ptrs.ptr, capi.i64(fff.shape[1]), capi.vp(fff),
                   capi.i64(space.n_nodes), capi.i64(dirichlet.numel()), capi.vp(dirichlet),
                   keep=(ctx, space, fff, dirichlet))


def elasticity_op(ctx, space: SSMeshDevice, adj, det, mu, lam, dirichlet, dtype, tensor_cores=False) -> Handle:
    """Linear-elasticity operator.  ``tensor_cores`` (float32 only) runs the element
    contraction in BF16 on the tensor cores: fast but accurate to about 1e-2 of
    |K||u| per entry, so it is meant for multigrid smoothers, not for a Krylov
    operator."""
    E = space.n_elements
    rt = rt_of(dtype)
    if tensor_cores:
        if rt != capi.FLOAT32:
            raise ValueError("tensor-core elasticity contraction needs float32 vectors")
        rt = capi.FLOAT32_BF16TC
    return _create(_lib().sfem_gb300_elasticity_op_create, ctx.ptr, c_int(rt), c_int(space.element_type),
                   capi.i64(E), space.elements_ptrs.ptr, capi.i64(adj.shape[1]), capi.vp(adj), capi.vp(det),
                   c_double(mu), c_double(lam), capi.i64(space.n_nodes), capi.i64(dirichlet.numel()),
                   capi.vp(dirichlet), keep=(ctx, space, adj, det, dirichlet))


def prolongation_op(ctx, coarse: SSMeshDevice, fine: SSMeshDevice, vec, dirichlet_fine, dtype) -> Handle:
    return _create(_lib().sfem_gb300_prolongation_op_create, ctx.ptr, c_int(rt_of(dtype)), capi.i64(fine.n_elements),
                   c_int(coarse.level), coarse.lidx_ptrs.ptr, capi.i64(coarse.n_nodes), c_int(fine.level),
                   fine.lidx_ptrs.ptr, capi.i64(fine.n_nodes), c_int(vec), capi.i64(dirichlet_fine.numel()),
                   capi.vp(dirichlet_fine), keep=(ctx, coarse, fine, dirichlet_fine))


def restriction_op(ctx, fine: SSMeshDevice, coarse: SSMeshDevice, vec, dirichlet_coarse, dtype) -> Handle:
    return _create(_lib().sfem_gb300_restriction_op_create, ctx.ptr, c_int(rt_of(dtype)), capi.i64(fine.n_elements),
                   c_int(fine.level), fine.lidx_ptrs.ptr, capi.vp(fine.count), capi.i64(fine.n_nodes),
                   c_int(coarse.level), coarse.lidx_ptrs.ptr, capi.i64(coarse.n_nodes), c_int(vec),
                   capi.i64(dirichlet_coarse.numel()), capi.vp(dirichlet_coarse), keep=(ctx, coarse, fine, dirichlet_coarse))


def jacobi(ctx, diag, relaxation=1.0) -> Handle:
    return _create(_lib().sfem_gb300_jacobi_create, ctx.ptr, c_int(rt_of(diag.dtype)), capi.i64(diag.numel()),
                   capi.vp(diag), c_double(relaxation), keep=(ctx,))


def block_jacobi(ctx, inv_block6) -> Handle:
    return _create(_lib().sfem_gb300_block_jacobi_create, ctx.ptr, c_int(rt_of(inv_block6.dtype)),
                   capi.i64(inv_block6.numel() // 6), capi.vp(inv_block6), keep=(ctx, inv_block6))


def stationary(ctx, op, precond, max_it) -> Handle:
    return _create(_lib().sfem_gb300_stationary_create, ctx.ptr, op.ptr, precond.ptr, c_int(max_it),
                   keep=(ctx, op, precond))


def chebyshev3(ctx, op, max_it=2, scale_eig_max=1.02, scale_eig_min=0.06, eigen_max_it=100, eigen_tol=1e-5,
               eig_max=None, inv_diag=None) -> Handle:
    h = _create(_lib().sfem_gb300_chebyshev3_create, ctx.ptr, op.ptr, capi.vp(inv_diag), c_int(max_it),
                c_double(scale_eig_max), c_double(scale_eig_min), c_int(eigen_max_it if eig_max is None else 1),
                c_double(eigen_tol), keep=(ctx, op, inv_diag))
    if eig_max is not None:
        capi.check(_lib().sfem_gb300_chebyshev3_set_eig_max(h.ptr, c_double(eig_max)), "set_eig_max")
    return h


def eig_max(cheb: Handle) -> float:
    v = c_double(0)
    capi.check(_lib().sfem_gb300_chebyshev3_eig_max(cheb.ptr, C.byref(v)), "eig_max")
    return v.value


RANDOM_SEED = 0x5EED5EED  # start vector of the power method (sfem_gb300_random_uniform)


def cg(ctx, op, precond=None, max_it=10000, rtol=1e-10, atol=0.0, residual_norm=False, flexible=False,
       check_every=1) -> Handle:
    h = _create(_lib().sfem_gb300_cg_create, ctx.ptr, op.ptr, precond.ptr if precond else None, c_int(max_it),
                c_double(rtol), c_double(atol), keep=(ctx, op, precond))
    if residual_norm or flexible or check_every != 1:
        capi.check(_lib().sfem_gb300_cg_set_options(h.ptr, int(residual_norm), int(flexible), int(check_every)),
                   "cg_set_options")
    return h


def multigrid(ctx, dtype, max_it=1, cycle_type=1) -> Handle:
    return _create(_lib().sfem_gb300_mg_create, ctx.ptr, c_int(rt_of(dtype)), c_int(max_it), c_int(cycle_type),
                   keep=(ctx,))


def mg_add_level(mg, op, smoother, prolongation=None, restriction=None):
    capi.check(_lib().sfem_gb300_mg_add_level(mg.ptr, op.ptr, smoother.ptr, prolongation.ptr if prolongation else None,
                                              restriction.ptr if restriction else None), "mg_add_level")
    mg.keep += [op, smoother, prolongation, restriction]


def dense_solver(ctx, op) -> Handle:
    """Dense Cholesky-inverse solve of a small SPD operator (<= 1536 unknowns)."""
    return _create(_lib().sfem_gb300_dense_solver_create, ctx.ptr, op.ptr, keep=(ctx, op))


def mg_set_graph(mg, enable=True):
    capi.check(_lib().sfem_gb300_mg_set_graph(mg.ptr, int(enable)), "mg_set_graph")


DENSE_MAX = 1536


def mixed_precond(ctx, inner32) -> Handle:
    """Double-precision preconditioner z = |r| inner32(r / |r|) (e.g. a float multigrid
    V-cycle under a double flexible CG)."""
    return _create(_lib().sfem_gb300_mixed_precond_create, ctx.ptr, inner32.ptr, keep=(ctx, inner32))


def iterative_refinement(ctx, op64, inner32, max_it=50, rtol=1e-10) -> Handle:
    return _create(_lib().sfem_gb300_ir_create, ctx.ptr, op64.ptr, inner32.ptr, c_int(max_it), c_double(rtol),
                   keep=(ctx, op64, inner32))


# ---------------------------------------------------------------------------
# hierarchy builders
# ---------------------------------------------------------------------------
class CoarseSpaceDevice:
    """A :class:`CoarseHex8Level` resident on the GPU: its hex8 operator data and the
    CSR transfers to / from the next finer level."""

    is_macro_coarse = True

    def __init__(self, lvl: CoarseHex8Level, device):
        import torch

        self.lvl = lvl
        self.level = 1
        self.element_type = capi.HEX8
        self.n_elements = lvl.n_elements
        self.n_nodes = lvl.n_nodes
        self.n_fine_nodes = lvl.n_fine_nodes
        self.device = torch.device(device)
        t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(self.device)
        self.elements = t(lvl.hex8)
        self.elements_ptrs = capi.DevicePtrArray(self.elements)
        self.corners_ptrs = self.elements_ptrs
        self.points = t(lvl.points)
        self.points_ptrs = capi.DevicePtrArray(self.points)
        self.P = tuple(t(a) for a in lvl.P)  # finer rows x coarse cols
        self.R = tuple(t(a) for a in lvl.R)  # coarse rows x finer cols

    def dirichlet_nodes(self, faces=("x0",)):
        import torch

        ids = np.unique(np.concatenate([self.lvl.boundary_nodes(f) for f in faces])).astype(np.int32)
        return torch.from_numpy(ids).to(self.device)


def crs_transfer_op(ctx, csr, nrows, ncols, vec, dirichlet_out, dtype) -> Handle:
    """y = M x for a CSR (rowptr, colidx, weights) device triple; output Dirichlet dofs zeroed."""
    rp, ci, w = csr
    return _create(_lib().sfem_gb300_crs_transfer_op_create, ctx.ptr, c_int(rt_of(dtype)), capi.i64(nrows),
                   capi.i64(ncols), capi.vp(rp), capi.vp(ci), capi.vp(w), c_int(vec), capi.i64(dirichlet_out.numel()),
                   capi.vp(dirichlet_out), keep=(ctx, rp, ci, w, dirichlet_out))


class Hierarchy:
    """Device data of every level of a multigrid hierarchy on an :class:`SSMesh`
    (shared by both precisions): the sshex8 derefinement levels and, with
    ``coarsen_macro``, plain hex8 levels below the macro mesh
    (:func:`sfem_gb300.mesh.macro_coarse_levels`).

    Every space carries its own geometry (``fff``, ``adj``, ``det``); the sshex8
    levels share the macro element metric.  A per-macro-element ``coefficient``
    scales the metric; coarse hex8 levels take the mean over their 2x2x2 children."""

    def __init__(self, mesh: SSMesh, dirichlet_faces=("x0",), device="cuda:0", vec=1, coefficient=None,
                 coarsen_macro=False, min_coarse_nodes=64):
        import torch

        self.mesh = mesh
        self.vec = vec
        self.device = torch.device(device)
        self.spaces = [SSMeshDevice(mesh, l, device=self.device) for l in mesh.levels]
        for sp in self.spaces:
            lid = mesh.elements(sp.level)
            sp.lidx_elements = torch.from_numpy(np.ascontiguousarray(lid)).to(self.device)
            sp.lidx_ptrs = capi.DevicePtrArray(sp.lidx_elements)
            cnt = np.bincount(lid.reshape(-1), minlength=mesh.n_nodes(sp.level)).astype(np.uint16)
            sp.count = torch.from_numpy(cnt.view(np.int16)).to(self.device)
        self.n_sshex8_levels = len(self.spaces)
        self.coarse_levels = macro_coarse_levels(mesh, min_coarse_nodes) if coarsen_macro else []
        self.spaces += [CoarseSpaceDevice(lvl, self.device) for lvl in self.coarse_levels]
        self.dirichlet = [sp.dirichlet_nodes(dirichlet_faces) if dirichlet_faces else
                          torch.zeros(0, dtype=torch.int32, device=self.device) for sp in self.spaces]
        # geometry: one metric / adjugate per macro element for all sshex8 levels
        lap = Laplacian(self.spaces[0], coefficient=coefficient, packed=False).initialize()
        self.fff = lap.fff
        self.adj, self.det = self._adjugate(self.spaces[0])
        for sp in self.spaces[:self.n_sshex8_levels]:
            sp.fff, sp.adj, sp.det = self.fff, self.adj, self.det
        k = None if coefficient is None else np.asarray(coefficient, dtype=np.float64).reshape(mesh.nz, mesh.ny, mesh.nx)
        for sp in self.spaces[self.n_sshex8_levels:]:
            if k is not None:
                cx, cy, cz = sp.lvl.shape
                k = coarsen_coefficient(k, (cz, cy, cx))
            sp.fff = Laplacian(sp, coefficient=None if k is None else k.reshape(-1), packed=False).initialize().fff
            sp.adj, sp.det = self._adjugate(sp)

    def _adjugate(self, sp):
        import torch

        E = sp.n_elements
        adj = torch.empty((9, E), dtype=torch.float32, device=self.device)
        det = torch.empty(E, dtype=torch.float32, device=self.device)
        capi.check(capi.load().sfem_gb300_hex8_adjugate_fill(capi.i64(E), sp.corners_ptrs.ptr, sp.points_ptrs.ptr,
                                                            capi.i64(E), capi.vp(adj), capi.vp(det), None),
                   "adjugate_fill")
        return adj, det

    def n_dofs(self, k=0):
        return self.vec * self.spaces[k].n_nodes


def transfer_ops(ctx, H: Hierarchy, k: int, vec: int, dtype):
    """(P, R) between level k+1 (coarse) and level k (fine) of ``H``."""
    C_, F = H.spaces[k + 1], H.spaces[k]
    if getattr(C_, "is_macro_coarse", False):
        P = crs_transfer_op(ctx, C_.P, F.n_nodes, C_.n_nodes, vec, H.dirichlet[k], dtype)
        R = crs_transfer_op(ctx, C_.R, C_.n_nodes, F.n_nodes, vec, H.dirichlet[k + 1], dtype)
        return P, R
    return (prolongation_op(ctx, C_, F, vec, H.dirichlet[k], dtype),
            restriction_op(ctx, F, C_, vec, H.dirichlet[k + 1], dtype))


def build_poisson_mg(ctx, H: Hierarchy, dtype, smoother="chebyshev3", sweeps=2, coarse_rtol=1e-6, coarse_max_it=10000,
                     eig_max=None, jacobi_sweeps=3, coarse_check_every=10, eigen_max_it=30, coarse="cg", graph=False):
    """Geometric multigrid for the Laplacian on every level of ``H`` (one V-cycle per apply).

    coarse="cg": Jacobi-PCG to coarse_rtol on the coarsest level; coarse="dense": dense
    Cholesky-inverse solve (coarsest level <= 1536 unknowns).  graph=True replays the
    V-cycle as a CUDA graph (needs coarse="dense")."""
    import torch

    ops, smoothers, Ps, Rs = [], [], [], []
    nlev = len(H.spaces)
    eigs = []
    for k, sp in enumerate(H.spaces):
        op = laplacian_op(ctx, sp, sp.fff, H.dirichlet[k], dtype)
        ops.append(op)
        lap = Laplacian(sp, packed=False).set_fff(sp.fff)
        diag = torch.zeros(sp.n_nodes, dtype=dtype, device=H.device)
        lap.hessian_diag(diag)
        diag[H.dirichlet[k].long()] = 1
        if k == nlev - 1:
            if coarse == "dense":
                smoothers.append(dense_solver(ctx, op))
            else:
                jac = jacobi(ctx, diag, 1.0)
                smoothers.append(cg(ctx, op, jac, max_it=coarse_max_it, rtol=coarse_rtol,
                                    check_every=coarse_check_every))
        elif smoother in ("chebyshev3", "chebyshev3_plain"):
            em = None if eig_max is None else eig_max[k]
            inv = None
            if smoother == "chebyshev3":  # Jacobi-scaled Chebyshev (iteration on D^-1 A)
                inv = 1.0 / diag
            ch = chebyshev3(ctx, op, max_it=sweeps, eig_max=em, inv_diag=inv, eigen_max_it=eigen_max_it)
            eigs.append(globals()["eig_max"](ch))
            smoothers.append(ch)
        else:
            jac = jacobi(ctx, diag, 1.0)
            smoothers.append(stationary(ctx, op, jac, jacobi_sweeps))
    mg = multigrid(ctx, dtype)
    for k in range(nlev):
        P, R = transfer_ops(ctx, H, k, 1, dtype) if k + 1 < nlev else (None, None)
        mg_add_level(mg, ops[k], smoothers[k], P, R)
    mg.keep += [H]
    mg.eigs = eigs
    mg.smoothers = smoothers
    if graph:
        mg_set_graph(mg, True)
    return mg, ops[0]


def _elasticity_diag(H: Hierarchy, k, dtype, mu, lam):
    import torch

    sp = H.spaces[k]
    E = sp.n_elements
    d3 = torch.zeros(3 * sp.n_nodes, dtype=dtype, device=H.device)
    capi.check(capi.load().sfem_gb300_linear_elasticity_block_diag(
        sp.element_type, capi.i64(E), sp.elements_ptrs.ptr, capi.i64(E), capi.vp(sp.adj), capi.vp(sp.det), c_double(mu),
        c_double(lam), rt_of(dtype), capi.vp(d3), None, None), "elasticity diag")
    dn = H.dirichlet[k].long()
    for c in range(3):
        d3[3 * dn + c] = 1
    return d3


def build_elasticity_mg(ctx, H: Hierarchy, dtype, mu=1.0, lam=10.0, sweeps=2, coarse_rtol=1e-6,
                        coarse_max_it=10000, eig_max=None, coarse_check_every=10, eigen_max_it=30, scale_eig_max=1.1,
                        tensor_cores=False, coarse="cg", graph=False):
    """Geometric multigrid for linear elasticity (3 dofs / node) on every level of ``H``:
    Jacobi-scaled Chebyshev3 smoothing, nested vector transfer, Jacobi-PCG coarse solve
    (cf. the vector branch of algebra/mg/sfem_GeometricMultigrid.cpp:89-144).

    With ``tensor_cores`` (float32) the smoothers and the multigrid residuals of
    the non-coarsest levels use the BF16 tensor-core contraction; the coarse
    solve and the returned fine operator (for the outer Krylov method) stay
    FP32 SIMT."""
    ops, smoothers = [], []
    nlev = len(H.spaces)
    eigs = []
    fine_op = None
    for k, sp in enumerate(H.spaces):
        op = elasticity_op(ctx, sp, sp.adj, sp.det, mu, lam, H.dirichlet[k], dtype)
        if k == 0:
            fine_op = op
        if tensor_cores and k < nlev - 1:
            op = elasticity_op(ctx, sp, sp.adj, sp.det, mu, lam, H.dirichlet[k], dtype, tensor_cores=True)
        ops.append(op)
        d3 = _elasticity_diag(H, k, dtype, mu, lam)
        if k == nlev - 1:
            if coarse == "dense":
                smoothers.append(dense_solver(ctx, op))
            else:
                smoothers.append(cg(ctx, op, jacobi(ctx, d3, 1.0), max_it=coarse_max_it, rtol=coarse_rtol,
                                    check_every=coarse_check_every))
        else:
            em = None if eig_max is None else eig_max[k]
            ch = chebyshev3(ctx, op, max_it=sweeps, eig_max=em, inv_diag=1.0 / d3, eigen_max_it=eigen_max_it,
                            scale_eig_max=scale_eig_max)
            eigs.append(globals()["eig_max"](ch))
            smoothers.append(ch)
    mg = multigrid(ctx, dtype)
    for k in range(nlev):
        P, R = transfer_ops(ctx, H, k, 3, dtype) if k + 1 < nlev else (None, None)
        mg_add_level(mg, ops[k], smoothers[k], P, R)
    mg.keep += [H, fine_op]
    mg.eigs = eigs
    if graph:
        mg_set_graph(mg, True)
    return mg, fine_op


class CompensatedResidual:
    """r = b - A x of the finest level's FP64 operator with A x accumulated in
    double-double (``sfem_gb300_residual_dd``): the residual of an FP64 iterate to
    about 1e-30 relative to (|A||x|)_i, where a plain FP64 evaluation is limited to
    about 1e-16 (|A||x|)_i.  kind: "laplacian" (the hierarchy's FFF, coefficient
    included) or "elasticity" (mu, lam)."""

    def __init__(self, H: Hierarchy, kind="laplacian", mu=1.0, lam=10.0):
        import torch

        sp = H.spaces[0]
        E = sp.n_elements
        lib = _lib()
        self.space, self.dirichlet = sp, H.dirichlet[0]
        self.bs = 3 if kind == "elasticity" else 1
        ne = 8 * self.bs
        self.em = torch.empty(E * ne * ne, dtype=torch.float64, device=H.device)
        if kind == "elasticity":
            capi.check(lib.sfem_gb300_linear_elasticity_element_matrices(
                sp.element_type, capi.i64(E), capi.i64(H.adj.shape[1]), capi.vp(H.adj), capi.vp(H.det),
                c_double(mu), c_double(lam), capi.FLOAT64, capi.vp(self.em), None), "element matrices")
        else:
            capi.check(lib.sfem_gb300_sshex8_laplacian_element_matrix(
                sp.element_type, capi.i64(E), capi.i64(H.fff.shape[1]), capi.vp(H.fff), capi.FLOAT64,
                capi.vp(self.em), None), "element matrices")
        # hex8 levels keep their corners in hex8 order; sshex8 levels in lidx order
        self.elements = sp.elements_ptrs
        self.n = self.bs * sp.n_nodes
        self.work = torch.empty(2 * self.n, dtype=torch.float64, device=H.device)

    def __call__(self, x, b, r=None, x_lo=None):
        """b - A (x + x_lo) (x_lo: the low part of a double-double solution, or None)."""
        import torch

        r = torch.empty_like(b) if r is None else r
        capi.check(_lib().sfem_gb300_residual_dd(
            self.space.element_type, c_int(self.bs), capi.i64(self.space.n_elements), self.elements.ptr,
            capi.vp(self.em), capi.i64(self.n), capi.vp(x), capi.vp(x_lo), capi.vp(b),
            capi.i64(self.dirichlet.numel()), capi.vp(self.dirichlet), capi.vp(self.work), capi.vp(r), None),
            "sfem_gb300_residual_dd")
        return r

    def relative(self, x, b, x_lo=None):
        import torch

        r = self(x, b, x_lo=x_lo)
        return float(torch.linalg.vector_norm(r) / torch.linalg.vector_norm(b))


def dd_axpy(alpha, e, x_hi, x_lo):
    """(x_hi, x_lo) += alpha e, error-free (the solution of a refinement kept in double-double)."""
    capi.check(_lib().sfem_gb300_dd_axpy(capi.i64(e.numel()), c_double(alpha), capi.vp(e), capi.vp(x_hi),
                                         capi.vp(x_lo), None), "sfem_gb300_dd_axpy")
