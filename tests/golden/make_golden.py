"""Generate tests/golden/*.npz from the reference's own CPU kernels.

Run where the reference tree is present (it builds oracle/_ref/libsfem_ref.so
from the reference sources in place).  The fixtures pin the oracle
restatement on machines without the reference tree.

    python tests/golden/make_golden.py
"""

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

import oracle as O  # noqa: E402
from sfem_gb300.mesh import SSMesh  # noqa: E402

OUT = Path(__file__).resolve().parent


def main():
    assert O.ref() is not None, "reference kernels unavailable"
    rng = np.random.default_rng(20261203)
    # sshex8 L=4 on a perturbed 2x2x1 macro mesh of [0,2]x[0,1]x[0,1]
    L = 4
    m = SSMesh(2, 2, 1, L, box=((0, 2), (0, 1), (0, 1)), perturb=0.15, seed=11)
    el = m.elements(L)
    corners = el[m.macro_corner_lidx(L)]
    fff = O.fff_fill(corners, m.points, use_ref=True)
    adj, det = O.adjugate_fill(corners, m.points, use_ref=True)
    n = m.n_nodes(L)
    x = rng.standard_normal(n)
    u = rng.standard_normal(3 * n)
    lap = O.sshex8_laplacian_apply(L, el, fff, x, use_ref=True)
    ela = O.linear_elasticity_apply(L, el, adj, det, 1.0, 10.0, u, use_ref=True)
    e2 = m.elements(2)
    n2 = m.n_nodes(2)
    xc = rng.standard_normal(n2)
    prol = O.prolongate(2, e2, L, el, 1, xc, n, use_ref=True)
    cnt = O.incidence_count(L, el, n, use_ref=True)
    rest = O.restrict(L, el, cnt, 2, e2, 1, x, n2, use_ref=True)
    e1 = m.elements(1)
    n1 = m.n_nodes(1)
    x1 = rng.standard_normal(n1)
    hprol = O.prolongate(1, e1, 2, e2, 1, x1, n2, use_ref=True)
    cnt2 = O.incidence_count(2, e2, n2, use_ref=True)
    hrest = O.restrict(2, e2, cnt2, 1, e1, 1, xc, n1, use_ref=True)
    h8 = m.hex8_elements()
    hlap = O.hex8_laplacian_apply(h8, fff, x1, use_ref=True)
    A = O.laplacian_matrix(fff[0].astype(np.float64) / L, use_ref=True)
    K = O.elasticity_matrix(1.0, 10.0, adj[0].astype(np.float64) / L**2, float(det[0]) / L**3, use_ref=True)
    np.savez_compressed(
        OUT / "sshex8_L4_2x2x1.npz",
        nx=2, ny=2, nz=1, level=L, box=np.array([[0, 2], [0, 1], [0, 1]], float), perturb=0.15, seed=11,
        elements=el, points=m.points, fff=fff, adjugate=adj, determinant=det, x=x, u=u, laplacian_apply=lap,
        elasticity_apply=ela, mu=1.0, lam=10.0, x_coarse2=xc, prolongate_2_4=prol, count_4=cnt, restrict_4_2=rest,
        x_level1=x1, prolongate_1_2=hprol, count_2=cnt2, restrict_2_1=hrest, hex8_elements=h8,
        hex8_laplacian_apply=hlap, laplacian_matrix_e0=A, elasticity_matrix_e0=K)
    print("wrote", OUT / "sshex8_L4_2x2x1.npz")
    # levels without a compile-time GPU kernel: Laplacian and elasticity at L = 5, 12, 16,
    # transfers between 8 and 16
    out = {}
    for L, n, seed in ((5, (2, 1, 1), 21), (12, (1, 1, 1), 22), (16, (1, 1, 1), 23)):
        m = SSMesh(*n, L, box=((0, n[0]), (0, 1), (0, 1)), perturb=0.15, seed=seed)
        el = m.elements(L)
        corners = el[m.macro_corner_lidx(L)]
        fff = O.fff_fill(corners, m.points, use_ref=True)
        adj, det = O.adjugate_fill(corners, m.points, use_ref=True)
        nn = m.n_nodes(L)
        x = rng.standard_normal(nn)
        u = rng.standard_normal(3 * nn)
        out.update({f"L{L}_elements": el, f"L{L}_points": m.points, f"L{L}_fff": fff, f"L{L}_adjugate": adj,
                    f"L{L}_determinant": det, f"L{L}_x": x, f"L{L}_u": u,
                    f"L{L}_laplacian_apply": O.sshex8_laplacian_apply(L, el, fff, x, use_ref=True),
                    f"L{L}_elasticity_apply": O.linear_elasticity_apply(L, el, adj, det, 1.0, 10.0, u, use_ref=True)})
        if L == 16:
            e8 = m.elements(8)
            n8 = m.n_nodes(8)
            x8 = rng.standard_normal(n8)
            cnt = O.incidence_count(16, el, nn, use_ref=True)
            out.update({"L16_elements8": e8, "L16_x8": x8,
                        "L16_prolongate_8_16": O.prolongate(8, e8, 16, el, 1, x8, nn, use_ref=True),
                        "L16_restrict_16_8": O.restrict(16, el, cnt, 8, e8, 1, x, n8, use_ref=True)})
    np.savez_compressed(OUT / "sshex8_high_levels.npz", mu=1.0, lam=10.0, **out)
    print("wrote", OUT / "sshex8_high_levels.npz")
    make_float32_stencil()
    make_coefficient()


def make_float32_stencil():
    """affine_sshex8_laplacian_stencil_apply_fff built in the reference's float32 number
    configuration (real, scalar, accumulator = float): the pin of the float32 stencil
    restatement and of the CPU baseline the benchmark times."""
    assert O.ref_f32() is not None, "reference kernels (float32 configuration) unavailable"
    rng = np.random.default_rng(20261204)
    out = {}
    for L, n, seed in ((4, (3, 2, 2), 31), (2, (2, 2, 2), 32), (5, (2, 1, 1), 33)):
        m = SSMesh(*n, L, box=((0, n[0]), (0, n[1]), (0, n[2])), perturb=0.15, seed=seed)
        el = m.elements(L)
        fff = O.fff_fill(el[m.macro_corner_lidx(L)], m.points, use_ref=True)
        x = rng.standard_normal(m.n_nodes(L)).astype(np.float32)
        out.update({f"L{L}_elements": el, f"L{L}_fff": fff, f"L{L}_x": x,
                    f"L{L}_apply_f32": O.sshex8_laplacian_stencil_apply_f32(L, el, fff, x, use_ref=True),
                    f"L{L}_apply_f64": O.sshex8_laplacian_apply(L, el, fff, x.astype(np.float64), use_ref=True)})
    np.savez_compressed(OUT / "sshex8_stencil_float32.npz", **out)
    print("wrote", OUT / "sshex8_stencil_float32.npz")


def make_coefficient():
    """The variable-coefficient operator of the learned-smoother workload: k = exp(g) per
    macro element folded into the FFF (FFF * k_e in float32), applied by the reference's
    affine_sshex8_laplacian_stencil_apply_fff -- exact for a per-macro-element coefficient."""
    from sfem_gb300.coefficients import lognormal_coefficient

    assert O.ref() is not None, "reference kernels unavailable"
    L = 4
    m = SSMesh(6, 5, 4, L, perturb=0.1, seed=41)
    el = m.elements(L)
    fff = O.fff_fill(el[m.macro_corner_lidx(L)], m.points, use_ref=True)
    k = lognormal_coefficient(6, 5, 4, ell=2.0, sigma=1.0, seed=42)
    fffk = (fff * k[:, None]).astype(np.float32)
    x = np.random.default_rng(43).standard_normal(m.n_nodes(L))
    y = O.sshex8_laplacian_apply(L, el, fffk, x, use_ref=True)
    np.savez_compressed(OUT / "sshex8_coefficient.npz", elements=el, fff=fff, k=k, fff_scaled=fffk, x=x,
                        laplacian_apply=y, nx=6, ny=5, nz=4, level=L, perturb=0.1, seed=41)
    print("wrote", OUT / "sshex8_coefficient.npz")


def make_nonaffine():
    """The non-affine sshex8 Laplacian: the reference's sshex8_laplacian_apply
    (operators/sshex8/sshex8_laplacian.cpp:39-182; six-point rule per micro element, FFF
    of the trilinear macro map at every point) on perturbed macro meshes at L = 2 and 4,
    and the reference's affine_sshex8_laplacian_apply (:184-330) on the same meshes."""
    assert O.ref() is not None, "reference kernels unavailable"
    out = {}
    for L, n, seed in ((2, (4, 3, 2), 51), (4, (3, 2, 2), 52)):
        m = SSMesh(*n, L, perturb=0.2, seed=seed)
        el = m.elements(L)
        x = np.random.default_rng(seed + 100).standard_normal(m.n_nodes(L))
        y = O.sshex8_laplacian_apply_nonaffine(L, el, m.points, x, use_ref=True)
        # the reference's affine form from the corner points (FFF at the element centre,
        # sshex8_laplacian.cpp:184-330) on the same mesh
        ya = O.sshex8_laplacian_apply_affine_points_ref(L, el, m.points, x)
        out.update({f"L{L}_elements": el, f"L{L}_points": m.points.astype(np.float32), f"L{L}_x": x,
                    f"L{L}_apply": y, f"L{L}_affine_apply": ya, f"L{L}_shape": np.array(n), f"L{L}_seed": seed})
    np.savez_compressed(OUT / "sshex8_nonaffine.npz", perturb=0.2, **out)
    print("wrote", OUT / "sshex8_nonaffine.npz")


if __name__ == "__main__":
    if len(sys.argv) > 1 and sys.argv[1] == "float32":
        make_float32_stencil()
    elif len(sys.argv) > 1 and sys.argv[1] == "coefficient":
        make_coefficient()
    elif len(sys.argv) > 1 and sys.argv[1] == "nonaffine":
        make_nonaffine()
    else:
        main()
