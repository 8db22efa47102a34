"""CPU tests: the oracle restatement is pinned against the reference's own CPU
kernels -- through the committed golden fixtures (always) and directly through
oracle/_ref when the reference tree is available."""

from pathlib import Path

import numpy as np
import pytest

import oracle as O
import oracle.solvers as OS
from sfem_gb300.mesh import SSMesh, derefinement_levels

GOLD = Path(__file__).resolve().parent / "golden" / "sshex8_L4_2x2x1.npz"


@pytest.fixture(scope="module")
def gold():
    return dict(np.load(GOLD))


def _rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def test_mesh_matches_golden(gold):
    m = SSMesh(2, 2, 1, 4, box=((0, 2), (0, 1), (0, 1)), perturb=0.15, seed=11)
    assert np.array_equal(m.elements(4), gold["elements"])
    assert np.array_equal(m.points, gold["points"])
    assert np.array_equal(m.hex8_elements(), gold["hex8_elements"])


def test_oracle_geometry_bitexact(gold):
    el = gold["elements"]
    m = SSMesh(2, 2, 1, 4, box=((0, 2), (0, 1), (0, 1)), perturb=0.15, seed=11)
    corners = el[m.macro_corner_lidx(4)]
    assert np.array_equal(O.fff_fill(corners, gold["points"]), gold["fff"])
    adj, det = O.adjugate_fill(corners, gold["points"])
    assert np.array_equal(adj, gold["adjugate"]) and np.array_equal(det, gold["determinant"])


def test_oracle_element_matrices(gold):
    A = O.laplacian_matrix(gold["fff"][0].astype(np.float64) / 4)
    assert _rel(A, gold["laplacian_matrix_e0"]) < 1e-14
    K = O.elasticity_matrix(1.0, 10.0, gold["adjugate"][0].astype(np.float64) / 16, float(gold["determinant"][0]) / 64)
    assert _rel(K, gold["elasticity_matrix_e0"]) < 1e-14
    assert np.abs(K - K.T).max() == 0


def test_oracle_applies(gold):
    el, fff = gold["elements"], gold["fff"]
    assert _rel(O.sshex8_laplacian_apply(4, el, fff, gold["x"]), gold["laplacian_apply"]) < 1e-14
    assert _rel(O.hex8_laplacian_apply(gold["hex8_elements"], fff, gold["x_level1"]), gold["hex8_laplacian_apply"]) < 1e-14
    ela = O.linear_elasticity_apply(4, el, gold["adjugate"], gold["determinant"], 1.0, 10.0, gold["u"])
    assert _rel(ela, gold["elasticity_apply"]) < 1e-14


def test_oracle_transfer(gold):
    m = SSMesh(2, 2, 1, 4, box=((0, 2), (0, 1), (0, 1)), perturb=0.15, seed=11)
    el, e2, e1 = m.elements(4), m.elements(2), m.elements(1)
    n, n2, n1 = m.n_nodes(4), m.n_nodes(2), m.n_nodes(1)
    assert np.array_equal(O.incidence_count(4, el, n), gold["count_4"])
    assert _rel(O.prolongate(2, e2, 4, el, 1, gold["x_coarse2"], n), gold["prolongate_2_4"]) < 1e-15
    assert _rel(O.restrict(4, el, gold["count_4"], 2, e2, 1, gold["x"], n2), gold["restrict_4_2"]) < 1e-14
    assert _rel(O.prolongate(1, e1, 2, e2, 1, gold["x_level1"], n2), gold["prolongate_1_2"]) < 1e-15
    assert _rel(O.restrict(2, e2, gold["count_2"], 1, e1, 1, gold["x_coarse2"], n1), gold["restrict_2_1"]) < 1e-14


def test_stencil_equals_element_matrix_on_skewed_hex():
    """Known answer (operators/stencil/tests/sfem_StencilTest.cpp:66-140): the reference's
    27-point stencil + surface pass equals the element-matrix apply on a skewed hex, L=16."""
    if O.ref() is None:
        pytest.skip("reference kernels unavailable")
    m = SSMesh(1, 1, 1, 16, perturb=0.0)
    # skew the single macro element
    pts = m.points.astype(np.float64)
    pts[0] += 0.3 * pts[1] + 0.1 * pts[2]
    pts[2] += 0.2 * pts[0]
    el = m.elements(16)
    fff = O.fff_fill(el[m.macro_corner_lidx(16)], pts.astype(np.float32))
    x = np.random.default_rng(0).standard_normal(m.n_nodes())
    a = O.sshex8_laplacian_apply(16, el, fff, x, use_ref=True)
    b = O.sshex8_laplacian_apply(16, el, fff, x)
    assert np.abs(a - b).max() < 1e-8


def test_operator_properties():
    """Laplacian rows sum to zero (A 1 = 0 without constraints); Galerkin consistency
    A_c 1 = P^T A P 1 (algebra/sfem_Multigrid.hpp:112-173) holds trivially for constants."""
    m = SSMesh(3, 2, 2, 4, perturb=0.1, seed=1)
    el = m.elements(4)
    fff = O.fff_fill(el[m.macro_corner_lidx(4)], m.points)
    ones = np.ones(m.n_nodes())
    assert np.abs(O.sshex8_laplacian_apply(4, el, fff, ones)).max() < 1e-12
    # symmetry: (A x, y) = (x, A y)
    rng = np.random.default_rng(0)
    x, y = rng.standard_normal(m.n_nodes()), rng.standard_normal(m.n_nodes())
    Ax, Ay = O.sshex8_laplacian_apply(4, el, fff, x), O.sshex8_laplacian_apply(4, el, fff, y)
    assert abs(Ax @ y - x @ Ay) < 1e-10 * abs(Ax @ y)


def test_reference_direct_pin():
    """Where the reference tree is present, pin the restatement against it on a fresh mesh."""
    if O.ref() is None:
        pytest.skip("reference kernels unavailable")
    m = SSMesh(3, 2, 2, 3, perturb=0.12, seed=5)
    el = m.elements(3)
    corners = el[m.macro_corner_lidx(3)]
    fff = O.fff_fill(corners, m.points, use_ref=True)
    x = np.random.default_rng(2).standard_normal(m.n_nodes())
    assert _rel(O.sshex8_laplacian_apply(3, el, fff, x), O.sshex8_laplacian_apply(3, el, fff, x, use_ref=True)) < 1e-14
    adj, det = O.adjugate_fill(corners, m.points, use_ref=True)
    u = np.random.default_rng(3).standard_normal(3 * m.n_nodes())
    assert _rel(O.linear_elasticity_apply(3, el, adj, det, 2.0, 3.0, u),
                O.linear_elasticity_apply(3, el, adj, det, 2.0, 3.0, u, use_ref=True)) < 1e-14


def test_derefinement_levels():
    assert derefinement_levels(4) == [4, 2, 1]
    assert derefinement_levels(3) == [3, 1]
    assert derefinement_levels(8) == [8, 4, 2, 1]
    assert derefinement_levels(6) == [6, 3, 1]
    assert derefinement_levels(1) == [1]


def test_nested_numbering_prefix():
    m = SSMesh(3, 2, 2, 4)
    for l in m.levels:
        assert m.elements(l).max() < m.n_nodes(l)
    # coarse level nodes are the same physical points as in the fine level
    e2, e4 = m.elements(2), m.elements(4)
    for lid2 in range(27):
        z, y, x = lid2 // 9, (lid2 // 3) % 3, lid2 % 3
        assert np.array_equal(e2[lid2], e4[z * 2 * 25 + y * 2 * 5 + x * 2])


def test_oracle_cg_converges():
    m = SSMesh(4, 4, 4, 1)
    el = m.hex8_elements()
    fff = O.fff_fill(el, m.points)
    dn = m.all_boundary_nodes(1)

    def apply(v):
        y = O.hex8_laplacian_apply(el, fff, v)
        y[dn] = v[dn]
        return y

    b = np.ones(m.n_nodes(1))
    b[dn] = 0
    x, it = OS.cg(apply, b, rtol=1e-12)
    assert np.linalg.norm(b - apply(x)) < 1e-10 * np.linalg.norm(b)


def test_patchconv_oracle_matches_torch_autograd():
    """The oracle loop nests of the learned-smoother network agree with an independent
    torch CPU conv3d + autograd (forward, input gradient, weight gradient)."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(0)
    for cin, cout in ((1, 16), (16, 16), (16, 1)):
        P = 3
        x = rng.standard_normal((P, 125, cin)).astype(np.float32)
        W = rng.standard_normal((cout, cin, 27)).astype(np.float32)
        xt = torch.from_numpy(x).double().reshape(P, 5, 5, 5, cin).permute(0, 4, 1, 2, 3).requires_grad_(True)
        Wt = torch.from_numpy(W).double().reshape(cout, cin, 3, 3, 3).requires_grad_(True)
        yt = torch.nn.functional.conv3d(xt, Wt, padding=1).permute(0, 2, 3, 4, 1).reshape(P, 125, cout)
        y = O.patchconv_forward(P, cin, cout, x, W, 0).reshape(P, 125, cout)
        assert np.abs(yt.detach().numpy() - y).max() < 1e-11
        g = rng.standard_normal((P, 125, cout)).astype(np.float32)
        yt.backward(torch.from_numpy(g).double())
        gin = O.patchconv_backward_data(P, cin, cout, g, W).reshape(P, 125, cin)
        assert np.abs(xt.grad.permute(0, 2, 3, 4, 1).reshape(P, 125, cin).numpy() - gin).max() < 1e-11
        dW = O.patchconv_backward_weights(P, cin, cout, g, x)
        assert np.abs(Wt.grad.reshape(-1).numpy() - dW).max() < 1e-11


def test_float32_configuration_apply():
    """The float32 restatement (reference number configuration SFEM_REAL_TYPE=float32)
    agrees with the FP64 apply to float rounding and keeps its symmetry."""
    from sfem_gb300.mesh import SSMesh

    L = 4
    m = SSMesh(3, 3, 2, L, perturb=0.1, seed=4)
    el = m.elements(L)
    fff = O.fff_fill(el[m.macro_corner_lidx(L)], m.points)
    rng = np.random.default_rng(2)
    x, z = rng.standard_normal(m.n_nodes()), rng.standard_normal(m.n_nodes())
    a = O.sshex8_laplacian_apply(L, el, fff, x)
    b = O.sshex8_laplacian_apply_f32(L, el, fff, x)
    assert b.dtype == np.float32
    assert np.abs(a - b).max() <= 1e-5 * np.abs(a).max()
    zb = O.sshex8_laplacian_apply_f32(L, el, fff, z)
    assert abs(float(z.astype(np.float32) @ b) - float(x.astype(np.float32) @ zb)) <= 1e-4 * abs(float(z @ a))


HIGH = Path(__file__).resolve().parent / "golden" / "sshex8_high_levels.npz"


@pytest.mark.parametrize("L", [5, 12, 16])
def test_oracle_matches_reference_golden_high_levels(L):
    """The oracle restatement at levels 5, 12 and 16 (the GPU's CTA-per-element kernels'
    reference) against outputs of the reference's own CPU kernels."""
    g = np.load(HIGH)
    el, fff, adj, det = g[f"L{L}_elements"], g[f"L{L}_fff"], g[f"L{L}_adjugate"], g[f"L{L}_determinant"]
    x, u = g[f"L{L}_x"], g[f"L{L}_u"]
    lap = O.sshex8_laplacian_apply(L, el, fff, x)
    ref = g[f"L{L}_laplacian_apply"]
    assert np.abs(lap - ref).max() <= 1e-13 * np.abs(ref).max()
    ela = O.linear_elasticity_apply(L, el, adj, det, float(g["mu"]), float(g["lam"]), u)
    ref = g[f"L{L}_elasticity_apply"]
    assert np.abs(ela - ref).max() <= 1e-13 * np.abs(ref).max()
    if L == 16:
        e8, x8 = g["L16_elements8"], g["L16_x8"]
        n = x.size
        prol = O.prolongate(8, e8, 16, el, 1, x8, n)
        assert np.abs(prol - g["L16_prolongate_8_16"]).max() <= 1e-14 * np.abs(prol).max()
        cnt = O.incidence_count(16, el, n)
        rest = O.restrict(16, el, cnt, 8, e8, 1, x, x8.size)
        assert np.abs(rest - g["L16_restrict_16_8"]).max() <= 1e-13 * np.abs(rest).max()


STENCIL_F32 = Path(__file__).resolve().parent / "golden" / "sshex8_stencil_float32.npz"


def test_stencil_form_matches_reference_golden(gold):
    """The node-centric (stencil) restatement of affine_sshex8_laplacian_stencil_apply_fff
    against that reference function's own FP64 output (L = 4 fixture) and the high-level
    fixtures (L = 5, 12, 16)."""
    lap = O.sshex8_laplacian_stencil_apply(4, gold["elements"], gold["fff"], gold["x"])
    assert _rel(lap, gold["laplacian_apply"]) < 1e-14
    g = np.load(HIGH)
    for L in (5, 12, 16):
        lap = O.sshex8_laplacian_stencil_apply(L, g[f"L{L}_elements"], g[f"L{L}_fff"], g[f"L{L}_x"])
        assert _rel(lap, g[f"L{L}_laplacian_apply"]) < 1e-14


@pytest.mark.parametrize("L", [2, 4, 5])
def test_stencil_form_float32_matches_reference_golden(L):
    """The float32 stencil restatement (the benchmark's CPU baseline) against the
    reference's stencil apply built with real_t = float, and the FP64 stencil apply
    against the reference's FP64 output on the same input."""
    g = np.load(STENCIL_F32)
    el, fff, x = g[f"L{L}_elements"], g[f"L{L}_fff"], g[f"L{L}_x"]
    y32 = O.sshex8_laplacian_stencil_apply_f32(L, el, fff, x)
    ref32 = g[f"L{L}_apply_f32"]
    assert y32.dtype == np.float32 and ref32.dtype == np.float32
    # float rounding in a different summation order: a few float ulps of the row scale
    assert np.abs(y32 - ref32).max() <= 2e-6 * np.abs(ref32).max()
    y64 = O.sshex8_laplacian_stencil_apply(L, el, fff, x.astype(np.float64))
    assert _rel(y64, g[f"L{L}_apply_f64"]) < 1e-14
    assert np.abs(ref32 - g[f"L{L}_apply_f64"]).max() <= 2e-6 * np.abs(ref32).max()


@pytest.mark.skipif(O.ref_f32() is None, reason="reference tree not present")
def test_stencil_form_float32_matches_reference_direct():
    """Directly against the reference's float32-configuration build on a fresh mesh."""
    m = SSMesh(3, 2, 2, 4, perturb=0.12, seed=9)
    el = m.elements(4)
    fff = O.fff_fill(el[m.macro_corner_lidx(4)], m.points)
    x = np.random.default_rng(5).standard_normal(m.n_nodes()).astype(np.float32)
    ref = O.sshex8_laplacian_stencil_apply_f32(4, el, fff, x, use_ref=True)
    ours = O.sshex8_laplacian_stencil_apply_f32(4, el, fff, x)
    assert np.abs(ours - ref).max() <= 2e-6 * np.abs(ref).max()


COEF = Path(__file__).resolve().parent / "golden" / "sshex8_coefficient.npz"


def test_variable_coefficient_matches_reference_golden():
    """k = exp(g) per macro element as FFF * k_e: the oracle's stencil apply on the scaled
    metric equals the reference's affine_sshex8_laplacian_stencil_apply_fff output."""
    g = np.load(COEF)
    fffk = (g["fff"] * g["k"][:, None]).astype(np.float32)
    assert np.array_equal(fffk, g["fff_scaled"])
    y = O.sshex8_laplacian_stencil_apply(4, g["elements"], fffk, g["x"])
    assert _rel(y, g["laplacian_apply"]) < 1e-14


NONAFFINE = Path(__file__).resolve().parent / "golden" / "sshex8_nonaffine.npz"


@pytest.mark.parametrize("L", [2, 4])
def test_nonaffine_laplacian_matches_reference_golden(L):
    """The non-affine sshex8 Laplacian restatement (six-point rule per micro element, FFF
    of the trilinear macro map) equals the reference's sshex8_laplacian_apply output on
    perturbed macro meshes, and differs from the affine (centre-FFF) form there."""
    g = np.load(NONAFFINE)
    el, pts, x = g[f"L{L}_elements"], g[f"L{L}_points"], g[f"L{L}_x"]
    y = O.sshex8_laplacian_apply_nonaffine(L, el, pts, x)
    assert _rel(y, g[f"L{L}_apply"]) < 1e-14
    aff = O.sshex8_laplacian_apply(L, el, O.fff_fill(el[SSMesh(*g[f"L{L}_shape"], L).macro_corner_lidx(L)], pts), x)
    assert _rel(aff, g[f"L{L}_apply"]) > 1e-3
    # the six-point face-centre rule is not exact for the Q1 stiffness integrand (degree 4
    # terms), so this form differs from the exact affine one even on affine meshes; it is
    # still a symmetric operator: (A x, z) = (x, A z)
    z = np.random.default_rng(6).standard_normal(x.shape[0])
    Az = O.sshex8_laplacian_apply_nonaffine(L, el, pts, z)
    assert abs(np.dot(y, z) - np.dot(x, Az)) < 1e-12 * np.abs(y).max() * np.abs(z).sum()


@pytest.mark.skipif(O.ref() is None, reason="reference tree not present")
def test_nonaffine_laplacian_matches_reference_directly():
    m = SSMesh(2, 3, 2, 3, perturb=0.25, seed=8)
    el = m.elements(3)
    x = np.random.default_rng(9).standard_normal(m.n_nodes(3))
    ours = O.sshex8_laplacian_apply_nonaffine(3, el, m.points, x)
    ref = O.sshex8_laplacian_apply_nonaffine(3, el, m.points, x, use_ref=True)
    assert _rel(ours, ref) < 1e-14


@pytest.mark.parametrize("L", [2, 4])
def test_affine_points_form_matches_reference_golden(L):
    """The reference's affine_sshex8_laplacian_apply (sshex8_laplacian.cpp:184-330: the
    metric computed from the corner points at the element centre, kept in double) and the
    affine form this library computes from the float32 FFF cache (the reference's default
    affine_sshex8_laplacian_stencil_apply_fff input) are the same operator: they agree to
    the float32 rounding of the metric (6e-8 relative), on perturbed meshes."""
    g = np.load(NONAFFINE)
    el, pts, x = g[f"L{L}_elements"], g[f"L{L}_points"], g[f"L{L}_x"]
    m = SSMesh(*g[f"L{L}_shape"], L)
    ours = O.sshex8_laplacian_stencil_apply(L, el, O.fff_fill(el[m.macro_corner_lidx(L)], pts), x)
    assert _rel(ours, g[f"L{L}_affine_apply"]) < 1e-7


def test_reference_root_is_explicit(tmp_path, monkeypatch):
    """The reference tree comes from an argument or SFEM_REFERENCE_ROOT, with a clear error
    when neither names an sfem checkout."""
    from oracle import build as ob

    monkeypatch.delenv("SFEM_REFERENCE_ROOT", raising=False)
    with pytest.raises(RuntimeError, match="SFEM_REFERENCE_ROOT"):
        ob.reference_root()
    with pytest.raises(RuntimeError, match="not an sfem tree"):
        ob.reference_root(str(tmp_path))
    (tmp_path / "operators" / "sshex8").mkdir(parents=True)
    (tmp_path / "operators" / "sshex8" / "sshex8_laplacian.cpp").write_text("")
    monkeypatch.setenv("SFEM_REFERENCE_ROOT", str(tmp_path))
    assert ob.reference_root() == tmp_path
