"""CPU oracle for the matrix-free operator path (TEST INFRASTRUCTURE ONLY).

Two libraries are exposed through ctypes:

* ``lib()``  -- the plain-C restatement ``oracle/src/oracle.c`` (always built);
* ``ref()``  -- the reference's own CPU sources compiled in place
  (``oracle/_ref/libsfem_ref.so``), available only where the reference tree is
  present; it pins the restatement.

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` may import this package.
"""

from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from . import build as _build

_lib = None
_ref = None
_ref_f32 = None

c_int = C.c_int
c_ptrdiff = C.c_ssize_t
c_double = C.c_double
c_void_p = C.c_void_p


def _ptr(a: np.ndarray):
    return C.c_void_p(a.ctypes.data)


class PtrArray:
    """``T**`` view of the rows of a 2-D C-contiguous array (keeps it alive)."""

    def __init__(self, a: np.ndarray):
        self.a = np.ascontiguousarray(a)
        n = self.a.shape[0]
        self.arr = (C.c_void_p * n)(*[self.a[i].ctypes.data for i in range(n)])

    @property
    def p(self):
        return C.cast(self.arr, C.c_void_p)


def lib():
    global _lib
    if _lib is None:
        path = _build.build_oracle()
        _lib = C.CDLL(str(path))
    return _lib


def ref():
    """The reference's compiled CPU kernels, or None when unavailable."""
    global _ref
    if _ref is None:
        path = _build.REF_LIB
        if not path.exists():
            try:
                path = _build.build_ref()
            except RuntimeError:  # no reference tree on this machine
                return None
        if path is None or not Path(path).exists():
            return None
        _ref = C.CDLL(str(path))
    return _ref


def ref_f32():
    """The reference's sshex8 Laplacian built in its float32 number configuration, or None."""
    global _ref_f32
    if _ref_f32 is None:
        path = _build.REF_LIB_F32
        if not path.exists():
            try:
                path = _build.build_ref_f32()
            except RuntimeError:  # no reference tree on this machine
                return None
        if path is None or not Path(path).exists():
            return None
        _ref_f32 = C.CDLL(str(path))
    return _ref_f32


# ---------------------------------------------------------------------------
# helpers (numpy in, numpy out)
# ---------------------------------------------------------------------------
def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def fff_fill(corners, points, use_ref=False):
    """FFF (AoS float32 [E,6]) at the element centre; ``corners`` int32 [8,E] in hex8 order."""
    L = ref() if use_ref else lib()
    fn = L.ref_hex8_fff_fill if use_ref else L.or_hex8_fff_fill
    E = corners.shape[1]
    out = np.zeros((E, 6), dtype=np.float32)
    ca, pa = PtrArray(corners.astype(np.int32)), PtrArray(_f32(points))
    fn(c_ptrdiff(E), ca.p, pa.p, _ptr(out))
    return out


def sshex8_laplacian_apply_nonaffine(L, elements, points, u, out=None, use_ref=False):
    """values += A u for the non-affine sshex8 Laplacian (six-point rule per micro element,
    FFF of the trilinear macro map at every point).  use_ref: the reference's own
    sshex8_laplacian_apply (operators/sshex8/sshex8_laplacian.cpp:39-182)."""
    E = elements.shape[1]
    u = _f64(u)
    out = np.zeros_like(u) if out is None else out
    ea, pa = PtrArray(elements.astype(np.int32)), PtrArray(_f32(points))
    if use_ref:
        rc = ref().sshex8_laplacian_apply(c_int(L), c_ptrdiff(E), ea.p, pa.p, _ptr(u), _ptr(out))
    else:
        rc = lib().or_sshex8_laplacian_apply_nonaffine(c_int(L), c_ptrdiff(E), ea.p, pa.p, _ptr(u), _ptr(out))
    assert rc == 0, rc
    return out


def sshex8_laplacian_apply_affine_points_ref(L, elements, points, u, out=None):
    """values += A u by the reference's affine_sshex8_laplacian_apply
    (operators/sshex8/sshex8_laplacian.cpp:184-330): the affine form with the metric
    computed from the corner points at the element centre (fixture generation only)."""
    E = elements.shape[1]
    u = _f64(u)
    out = np.zeros_like(u) if out is None else out
    ea, pa = PtrArray(elements.astype(np.int32)), PtrArray(_f32(points))
    rc = ref().affine_sshex8_laplacian_apply(c_int(L), c_ptrdiff(E), ea.p, pa.p, _ptr(u), _ptr(out))
    assert rc == 0, rc
    return out


def adjugate_fill(corners, points, use_ref=False):
    L = ref() if use_ref else lib()
    fn = L.ref_hex8_adjugate_and_det_fill if use_ref else L.or_hex8_adjugate_and_det_fill
    E = corners.shape[1]
    adj = np.zeros((E, 9), dtype=np.float32)
    det = np.zeros(E, dtype=np.float32)
    ca, pa = PtrArray(corners.astype(np.int32)), PtrArray(_f32(points))
    fn(c_ptrdiff(E), ca.p, pa.p, _ptr(adj), _ptr(det))
    return adj, det


def laplacian_matrix(fff6, use_ref=False):
    A = np.zeros(64)
    f = _f64(fff6)
    if use_ref:
        ref().ref_hex8_laplacian_matrix_fff_integral(_ptr(f), _ptr(A))
    else:
        lib().or_hex8_laplacian_matrix(_ptr(f), _ptr(A))
    return A.reshape(8, 8)


def elasticity_matrix(mu, lam, adj9, det, use_ref=False):
    K = np.zeros(576)
    a = _f64(adj9)
    if use_ref:
        ref().ref_hex8_linear_elasticity_matrix(c_double(mu), c_double(lam), _ptr(a), c_double(det), _ptr(K))
    else:
        lib().or_hex8_linear_elasticity_matrix(c_double(mu), c_double(lam), _ptr(a), c_double(det), _ptr(K))
    return K.reshape(24, 24)


def sshex8_laplacian_apply(L, elements, fff_aos, u, out=None, use_ref=False):
    """values += A u for the affine sshex8 Laplacian (float32 AoS FFF)."""
    E = elements.shape[1]
    u = _f64(u)
    out = np.zeros_like(u) if out is None else out
    ea = PtrArray(elements.astype(np.int32))
    f = _f32(fff_aos)
    if use_ref:
        ref().affine_sshex8_laplacian_stencil_apply_fff(c_int(L), c_ptrdiff(E), ea.p, _ptr(f), _ptr(u), _ptr(out))
    else:
        lib().or_sshex8_laplacian_apply(c_int(L), c_ptrdiff(E), ea.p, _ptr(f), _ptr(u), _ptr(out))
    return out


def sshex8_laplacian_apply_f32(L, elements, fff_aos, u, out=None):
    """values += A u in float32 arithmetic (the reference's float32 number configuration)."""
    E = elements.shape[1]
    u = np.ascontiguousarray(u, dtype=np.float32)
    out = np.zeros_like(u) if out is None else out
    assert out.dtype == np.float32
    ea = PtrArray(elements.astype(np.int32))
    f = _f32(fff_aos)
    lib().or_sshex8_laplacian_apply_f32(c_int(L), c_ptrdiff(E), ea.p, _ptr(f), _ptr(u), _ptr(out))
    return out


def sshex8_laplacian_stencil_apply(L, elements, fff_aos, u, out=None):
    """values += A u in the reference's node-centric stencil form (FP64)."""
    E = elements.shape[1]
    u = _f64(u)
    out = np.zeros_like(u) if out is None else out
    ea = PtrArray(elements.astype(np.int32))
    f = _f32(fff_aos)
    lib().or_sshex8_laplacian_stencil_apply(c_int(L), c_ptrdiff(E), ea.p, _ptr(f), _ptr(u), _ptr(out))
    return out


def sshex8_laplacian_stencil_apply_f32(L, elements, fff_aos, u, out=None, use_ref=False):
    """values += A u in the stencil form, float32 number configuration.  use_ref: the
    reference's own affine_sshex8_laplacian_stencil_apply_fff built with real_t = float."""
    E = elements.shape[1]
    u = np.ascontiguousarray(u, dtype=np.float32)
    out = np.zeros_like(u) if out is None else out
    assert out.dtype == np.float32
    ea = PtrArray(elements.astype(np.int32))
    f = _f32(fff_aos)
    if use_ref:
        ref_f32().affine_sshex8_laplacian_stencil_apply_fff(c_int(L), c_ptrdiff(E), ea.p, _ptr(f), _ptr(u),
                                                             _ptr(out))
    else:
        lib().or_sshex8_laplacian_stencil_apply_f32(c_int(L), c_ptrdiff(E), ea.p, _ptr(f), _ptr(u), _ptr(out))
    return out


def hex8_laplacian_apply(elements, fff_aos, u, out=None, use_ref=False):
    E = elements.shape[1]
    u = _f64(u)
    out = np.zeros_like(u) if out is None else out
    ea = PtrArray(elements.astype(np.int32))
    f = _f32(fff_aos)
    if use_ref:
        ref().hex8_laplacian_apply_opt(c_ptrdiff(E), ea.p, _ptr(f), _ptr(u), _ptr(out))
    else:
        lib().or_hex8_laplacian_apply(c_ptrdiff(E), ea.p, _ptr(f), _ptr(u), _ptr(out))
    return out


def laplacian_diag(L, elements, fff_aos, n, points=None, use_ref=False):
    """Operator diagonal.  L == 0 means plain hex8 (hex8 corner order)."""
    E = elements.shape[1]
    out = np.zeros(n)
    ea = PtrArray(elements.astype(np.int32))
    if use_ref:
        pa = PtrArray(_f32(points))
        if L == 0:
            ref().hex8_laplacian_diag(c_ptrdiff(E), c_ptrdiff(n), ea.p, pa.p, _ptr(out))
        else:
            ref().affine_sshex8_laplacian_diag(c_int(L), c_ptrdiff(E), ea.p, pa.p, _ptr(out))
    else:
        lib().or_laplacian_diag(c_int(L), c_ptrdiff(E), ea.p, _ptr(_f32(fff_aos)), _ptr(out))
    return out


def linear_elasticity_apply(L, elements, adj_aos, det, mu, lam, u, out=None, use_ref=False):
    """out += K u (interleaved xyz).  L == 0 means plain hex8 (hex8 corner order)."""
    E = elements.shape[1]
    u = _f64(u)
    out = np.zeros_like(u) if out is None else out
    ea = PtrArray(elements.astype(np.int32))
    a, d = _f32(adj_aos), _f32(det)
    if use_ref:
        if L == 0:
            raise NotImplementedError
        ref().affine_sshex8_linear_elasticity_apply_macro_adjugate(
            c_int(L), c_ptrdiff(E), c_ptrdiff(u.size // 3), ea.p, c_void_p(0), _ptr(a), _ptr(d), c_double(mu),
            c_double(lam), c_ptrdiff(3), C.c_void_p(u.ctypes.data), C.c_void_p(u.ctypes.data + 8),
            C.c_void_p(u.ctypes.data + 16), c_ptrdiff(3), C.c_void_p(out.ctypes.data),
            C.c_void_p(out.ctypes.data + 8), C.c_void_p(out.ctypes.data + 16))
    else:
        lib().or_linear_elasticity_apply(c_int(L), c_ptrdiff(E), ea.p, _ptr(a), _ptr(d), c_double(mu), c_double(lam),
                                         _ptr(u), _ptr(out))
    return out


def linear_elasticity_row_scale(L, elements, adj_aos, det, mu, lam, u):
    """sum_j |K_ij| |u_j| (element by element): the scale of per-entry parity checks."""
    E = elements.shape[1]
    u = np.abs(_f64(u))
    out = np.zeros_like(u)
    ea = PtrArray(elements.astype(np.int32))
    a, d = _f32(adj_aos), _f32(det)
    lib().or_linear_elasticity_apply_abs(c_int(L), c_ptrdiff(E), ea.p, _ptr(a), _ptr(d), c_double(mu),
                                         c_double(lam), _ptr(u), _ptr(out))
    return out


def linear_elasticity_block_diag(L, elements, adj_aos, det, mu, lam, n_nodes):
    E = elements.shape[1]
    d3 = np.zeros(3 * n_nodes)
    b6 = np.zeros(6 * n_nodes)
    ea = PtrArray(elements.astype(np.int32))
    lib().or_linear_elasticity_block_diag_sym(c_int(L), c_ptrdiff(E), ea.p, _ptr(_f32(adj_aos)), _ptr(_f32(det)),
                                             c_double(mu), c_double(lam), _ptr(d3), _ptr(b6))
    return d3, b6


def ref_linear_elasticity_diag(L, elements, points, mu, lam, n_nodes):
    E = elements.shape[1]
    out = np.zeros(3 * n_nodes)
    ea, pa = PtrArray(elements.astype(np.int32)), PtrArray(_f32(points))
    b = out.ctypes.data
    ref().affine_sshex8_linear_elasticity_diag(c_int(L), c_ptrdiff(E), c_ptrdiff(n_nodes), ea.p, pa.p, c_double(mu),
                                               c_double(lam), c_ptrdiff(3), c_void_p(b), c_void_p(b + 8),
                                               c_void_p(b + 16))
    return out


def ref_linear_elasticity_block_diag(L, elements, points, mu, lam, n_nodes):
    E = elements.shape[1]
    out = np.zeros(6 * n_nodes)
    ea, pa = PtrArray(elements.astype(np.int32)), PtrArray(_f32(points))
    b = out.ctypes.data
    ref().affine_sshex8_linear_elasticity_block_diag_sym(
        c_int(L), c_ptrdiff(E), c_ptrdiff(n_nodes), ea.p, pa.p, c_double(mu), c_double(lam), c_ptrdiff(6),
        *[c_void_p(b + 8 * k) for k in range(6)])
    return out


def incidence_count(L, elements, n, use_ref=False):
    E = elements.shape[1]
    out = np.zeros(n, dtype=np.uint16)
    ea = PtrArray(elements.astype(np.int32))
    if use_ref:
        ref().sshex8_element_node_incidence_count(c_int(L), c_int(1), c_ptrdiff(E), ea.p, _ptr(out))
    else:
        lib().or_incidence_count(c_int(L), c_ptrdiff(E), ea.p, _ptr(out))
    return out


def prolongate(from_level, from_elements, to_level, to_elements, vec, x_coarse, n_fine, use_ref=False):
    E = to_elements.shape[1]
    out = np.zeros(n_fine * vec)
    fa, ta = PtrArray(from_elements.astype(np.int32)), PtrArray(to_elements.astype(np.int32))
    xc = _f64(x_coarse)
    if use_ref:
        if from_level == 1:
            ref().sshex8_hierarchical_prolongation(c_int(to_level), c_ptrdiff(E), ta.p, c_int(vec), _ptr(xc), _ptr(out))
        else:
            ref().sshex8_prolongate(c_ptrdiff(E), c_int(from_level), c_int(1), fa.p, c_int(to_level), c_int(1), ta.p,
                                    c_int(vec), _ptr(xc), _ptr(out))
    else:
        rc = lib().or_sshex8_prolongate(c_ptrdiff(E), c_int(from_level), fa.p, c_int(to_level), ta.p, c_int(vec),
                                        _ptr(xc), _ptr(out))
        assert rc == 0
    return out


def restrict(from_level, from_elements, count, to_level, to_elements, vec, x_fine, n_coarse, use_ref=False):
    E = from_elements.shape[1]
    out = np.zeros(n_coarse * vec)
    fa, ta = PtrArray(from_elements.astype(np.int32)), PtrArray(to_elements.astype(np.int32))
    xf = _f64(x_fine)
    cnt = np.ascontiguousarray(count, dtype=np.uint16)
    if use_ref:
        if to_level == 1:
            ref().sshex8_hierarchical_restriction(c_int(from_level), c_ptrdiff(E), fa.p, _ptr(cnt), c_int(vec),
                                                  _ptr(xf), _ptr(out))
        else:
            ref().sshex8_restrict(c_ptrdiff(E), c_int(from_level), c_int(1), fa.p, _ptr(cnt), c_int(to_level), c_int(1),
                                  ta.p, c_int(vec), _ptr(xf), _ptr(out))
    else:
        rc = lib().or_sshex8_restrict(c_ptrdiff(E), c_int(from_level), fa.p, _ptr(cnt), c_int(to_level), ta.p,
                                      c_int(vec), _ptr(xf), _ptr(out))
        assert rc == 0
    return out


def crs_sym_spmv(rowptr, colidx, diag, offdiag, x):
    n = diag.size
    y = np.zeros(n)
    lib().or_crs_sym_spmv(c_ptrdiff(n), _ptr(np.ascontiguousarray(rowptr, np.int32)),
                          _ptr(np.ascontiguousarray(colidx, np.int32)), _ptr(_f64(diag)), _ptr(_f64(offdiag)),
                          _ptr(_f64(x)), _ptr(y))
    return y


def bsr_sym_spmv(bs, rowptr, colidx, diag_sym, offdiag, x):
    nb = rowptr.size - 1
    y = np.zeros(nb * bs)
    lib().or_bsr_sym_spmv(c_ptrdiff(nb), c_int(bs), _ptr(np.ascontiguousarray(rowptr, np.int32)),
                          _ptr(np.ascontiguousarray(colidx, np.int32)), _ptr(_f64(diag_sym)), _ptr(_f64(offdiag)),
                          _ptr(_f64(x)), _ptr(y))
    return y


def hex8_laplacian_crs_sym(elements, fff_aos, rowptr, colidx, n, use_ref=False, points=None):
    E = elements.shape[1]
    diag = np.zeros(n)
    off = np.zeros(colidx.size)
    ea = PtrArray(elements.astype(np.int32))
    rp, ci = np.ascontiguousarray(rowptr, np.int32), np.ascontiguousarray(colidx, np.int32)
    if use_ref:
        pa = PtrArray(_f32(points))
        ref().hex8_laplacian_crs_sym(c_ptrdiff(E), c_ptrdiff(n), ea.p, pa.p, _ptr(rp), _ptr(ci), _ptr(diag), _ptr(off))
    else:
        lib().or_hex8_laplacian_crs_sym(c_ptrdiff(E), ea.p, _ptr(_f32(fff_aos)), _ptr(rp), _ptr(ci), _ptr(diag),
                                        _ptr(off))
    return diag, off


# ---------------------------------------------------------------------------
# learned-smoother network (double-precision loop nests)
# ---------------------------------------------------------------------------
def patchconv_forward(P, cin, cout, x, W, relu):
    out = np.zeros(P * 125 * cout)
    lib().or_patchconv_forward(c_ptrdiff(P), c_int(cin), c_int(cout), _ptr(_f32(x)), _ptr(_f32(W)), c_int(relu),
                               _ptr(out))
    return out


def patchconv_backward_data(P, cin, cout, gout, W, in_act=None):
    out = np.zeros(P * 125 * cin)
    act = _f32(in_act) if in_act is not None else None
    lib().or_patchconv_backward_data(c_ptrdiff(P), c_int(cin), c_int(cout), _ptr(_f32(gout)), _ptr(_f32(W)),
                                     _ptr(act) if act is not None else c_void_p(0), _ptr(out))
    return out


def patchconv_backward_weights(P, cin, cout, gout, x):
    dW = np.zeros(cout * cin * 27)
    lib().or_patchconv_backward_weights(c_ptrdiff(P), c_int(cin), c_int(cout), _ptr(_f32(gout)), _ptr(_f32(x)),
                                        _ptr(dW))
    return dW


# ---------------------------------------------------------------------------
# compensated residuals and the CPU multigrid-CG solve
# ---------------------------------------------------------------------------
def laplacian_residual_dd(L, elements, fff_aos, x, b):
    """b - A x with A x summed in double-double (sshex8 L >= 2), rounded to double;
    constrained rows are left to the caller."""
    E = elements.shape[1]
    x, b = _f64(x), _f64(b)
    r = np.zeros_like(x)
    ea = PtrArray(elements.astype(np.int32))
    f = _f32(fff_aos)
    assert lib().or_sshex8_laplacian_residual_dd(c_int(L), c_ptrdiff(E), ea.p, _ptr(f), _ptr(x), _ptr(b),
                                                 c_ptrdiff(x.size), _ptr(r)) == 0
    return r


def elasticity_residual_dd(L, elements, adj_aos, det, mu, lam, x, b):
    """b - K x with K x summed in double-double (interleaved xyz), rounded to double."""
    E = elements.shape[1]
    x, b = _f64(x), _f64(b)
    r = np.zeros_like(x)
    ea = PtrArray(elements.astype(np.int32))
    a, d = _f32(adj_aos), _f32(det)
    assert lib().or_linear_elasticity_residual_dd(c_int(L), c_ptrdiff(E), ea.p, _ptr(a), _ptr(d), c_double(mu),
                                                  c_double(lam), _ptr(x), _ptr(b), c_ptrdiff(x.size), _ptr(r)) == 0
    return r


def residual_dd_em(bs, L, elements, em, x, b, x_lo=None):
    """b - A (x + x_lo) in double-double from given micro element matrices (the GPU's)."""
    E = elements.shape[1]
    x, b = _f64(x), _f64(b)
    r = np.zeros_like(x)
    ea = PtrArray(elements.astype(np.int32))
    em = _f64(em)
    xl = _f64(x_lo) if x_lo is not None else None
    assert lib().or_residual_dd_em(c_int(bs), c_int(L), c_ptrdiff(E), ea.p, _ptr(em), _ptr(x),
                                   _ptr(xl) if xl is not None else c_void_p(0), _ptr(b), c_ptrdiff(x.size),
                                   _ptr(r)) == 0
    return r


class _Level(C.Structure):
    _fields_ = [("L", c_int), ("elements", c_void_p), ("hex8_elements", c_void_p), ("n_nodes", c_ptrdiff),
                ("n_dirichlet", c_ptrdiff), ("dirichlet", c_void_p), ("count", c_void_p)]


class _Problem(C.Structure):
    _fields_ = [("kind", c_int), ("nelements", c_ptrdiff), ("geom", c_void_p), ("det", c_void_p), ("mu", c_double),
                ("lam", c_double), ("nlevels", c_int), ("levels", C.POINTER(_Level)), ("sweeps", c_int),
                ("scaled", c_int), ("scale_eig_max", c_double), ("coarse_rtol", c_double), ("rtol", c_double),
                ("max_it", c_int), ("flexible", c_int)]


class _Stats(C.Structure):
    _fields_ = [("iterations", c_int), ("restarts", c_int), ("coarse_iterations", c_int),
                ("true_rel_residual", c_double), ("setup_seconds", c_double), ("solve_seconds", c_double)]


def mg_pcg_solve(mesh, kind, b, dirichlet_faces=("x0",), geom=None, det=None, mu=1.0, lam=10.0, sweeps=2,
                 scaled=True, scale_eig_max=1.02, coarse_rtol=1e-8, rtol=1e-10, max_it=200, flexible=False):
    """CPU multigrid-preconditioned CG (oracle/src/solve.c) on the derefinement levels of an
    SSMesh (kind "laplacian" or "elasticity"); returns (x, stats dict).  geom: FFF AoS (or
    adjugate AoS with det) of the macro elements; computed here when omitted."""
    from sfem_gb300.mesh import derefinement_levels

    L = mesh.L
    keep = []
    levels = []
    for lv in derefinement_levels(L):
        el = mesh.elements(lv)
        pe = PtrArray(el.astype(np.int32))
        keep.append(pe)
        h8 = None
        if lv == 1:
            h8 = PtrArray(mesh.hex8_elements().astype(np.int32))
            keep.append(h8)
        n = mesh.n_nodes(lv)
        dn = np.unique(np.concatenate([mesh.boundary_nodes(f, lv) for f in dirichlet_faces])).astype(np.int32)
        cnt = incidence_count(lv, el, n)
        keep += [dn, cnt]
        levels.append(_Level(lv, pe.p.value, h8.p.value if h8 else None, n, dn.size, dn.ctypes.data,
                             cnt.ctypes.data))
    corners = mesh.elements(L)[mesh.macro_corner_lidx(L)]
    if kind == "laplacian":
        g = _f32(geom if geom is not None else fff_fill(corners, mesh.points))
        d = None
        k = 0
    else:
        if geom is None:
            geom, det = adjugate_fill(corners, mesh.points)
        g, d = _f32(geom), _f32(det)
        k = 1
    keep += [g, d]
    arr = (_Level * len(levels))(*levels)
    prob = _Problem(k, mesh.n_elements, g.ctypes.data, d.ctypes.data if d is not None else None, mu, lam,
                    len(levels), arr, sweeps, int(scaled), scale_eig_max, coarse_rtol, rtol, max_it, int(flexible))
    b = _f64(b)
    x = np.zeros_like(b)
    st = _Stats()
    rc = lib().or_mg_pcg_solve(C.byref(prob), _ptr(b), _ptr(x), C.byref(st))
    stats = {"rc": rc, "iterations": st.iterations, "restarts": st.restarts,
             "coarse_iterations": st.coarse_iterations, "true_rel_residual": st.true_rel_residual,
             "setup_seconds": st.setup_seconds, "solve_seconds": st.solve_seconds}
    return x, stats
