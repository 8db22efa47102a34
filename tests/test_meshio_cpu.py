"""Reference mesh folders and the semi-structured refinement of any hex8 mesh (CPU).

The fixture tests/golden/box_mesh_hex8/ was written by the reference's own
python/sfem/mesh/box_mesh.py (tests/golden/make_box_mesh.py).  The refinement is
checked against the structured generator: same nodes (matched by coordinates),
same nested level prefixes, same boundary sets and the same Laplacian apply
(oracle) -- also after renumbering the macro nodes and rotating every element's
corner order, which exercises the shared edge / face parameterisation.
"""

from pathlib import Path

import numpy as np
import pytest

import oracle as O
from sfem_gb300.mesh import HEX8_CORNERS, SSMesh
from sfem_gb300.meshio import (HexSSMesh, SfemMesh, format_meta, parse_meta, read_sfem_mesh, ssmesh_from_folder,
                               write_sfem_mesh)

FIXTURE = Path(__file__).resolve().parent / "golden" / "box_mesh_hex8"
FACES = {"left": "x0", "right": "x1", "bottom": "y0", "top": "y1", "back": "z0", "front": "z1"}


def test_read_reference_box_mesh():
    m = read_sfem_mesh(FIXTURE)
    assert m.element_type == "HEX8" and m.n_elements == 12 and m.n_nodes == 36
    p = m.points
    assert np.allclose(p.min(axis=1), 0) and np.allclose(p.max(axis=1), [2, 1, 1])
    # positive orientation: det J at the element centre
    for e in range(m.n_elements):
        X = p[:, m.elements[:, e]].T.astype(np.float64)
        J = np.zeros((3, 3))
        for c in range(8):
            s = np.where(HEX8_CORNERS[c] == 1, 0.25, -0.25)
            J += np.outer(X[c], s)
        assert np.linalg.det(J) > 0
    axis = {"left": (0, 0.0), "right": (0, 2.0), "bottom": (1, 0.0), "top": (1, 1.0), "back": (2, 0.0),
            "front": (2, 1.0)}
    for name, (d, v) in axis.items():
        assert np.array_equal(np.sort(m.boundary_nodes[name]), np.flatnonzero(np.isclose(p[d], v))), name


def _match(a_pts, b_pts):
    """perm with a_pts[:, i] == b_pts[:, perm[i]]."""
    ka = np.round(a_pts.T.astype(np.float64) * 1e4).astype(np.int64)
    kb = np.round(b_pts.T.astype(np.float64) * 1e4).astype(np.int64)
    ia = np.lexsort(ka.T[::-1])
    ib = np.lexsort(kb.T[::-1])
    assert np.array_equal(ka[ia], kb[ib]), "node coordinates differ"
    perm = np.empty(len(ka), dtype=np.int64)
    perm[ia] = ib
    return perm


def _compare_with_structured(hm: HexSSMesh, L: int, names=True):
    sm = SSMesh(3, 2, 2, L, box=((0, 2), (0, 1), (0, 1)))
    assert hm.levels == sm.levels
    perm = _match(hm.points, sm.points)
    for l in hm.levels:
        n = hm.n_nodes(l)
        assert n == sm.n_nodes(l)
        # nested prefixes: the level-l nodes are the same physical nodes
        assert (perm[:n] < n).all()
        el = hm.elements(l)
        assert el.shape == (sm.elements(l).shape[0], 12) and el.max() < n
    el_h, el_s = hm.elements(L), sm.elements(L)
    f_h = O.fff_fill(el_h[hm.macro_corner_lidx(L)], hm.points)
    f_s = O.fff_fill(el_s[sm.macro_corner_lidx(L)], sm.points)
    x_s = np.random.default_rng(0).standard_normal(sm.n_nodes(L))
    x_h = x_s[perm]
    y_s = O.sshex8_laplacian_apply(L, el_s, f_s, x_s) if L > 1 else O.hex8_laplacian_apply(el_s, f_s, x_s)
    y_h = O.sshex8_laplacian_apply(L, el_h, f_h, x_h) if L > 1 else O.hex8_laplacian_apply(el_h, f_h, x_h)
    assert np.abs(y_h - y_s[perm]).max() <= 1e-12 * np.abs(y_s).max()
    if names:
        for name, face in FACES.items():
            for l in hm.levels:
                got = np.sort(perm[hm.boundary_nodes(name, l)])
                assert np.array_equal(got, sm.boundary_nodes(face, l)), (name, l)


@pytest.mark.parametrize("L", [1, 2, 3, 4, 6])
def test_refined_reference_box_matches_structured(L):
    _compare_with_structured(ssmesh_from_folder(FIXTURE, L), L)


def _rotations():
    mats = []
    for perm in ([0, 1, 2], [0, 2, 1], [1, 0, 2], [1, 2, 0], [2, 0, 1], [2, 1, 0]):
        for signs in np.ndindex(2, 2, 2):
            R = np.zeros((3, 3), dtype=int)
            for i in range(3):
                R[i, perm[i]] = 1 if signs[i] == 0 else -1
            if round(np.linalg.det(R)) == 1:
                mats.append(R)
    assert len(mats) == 24
    return mats


@pytest.mark.parametrize("L", [2, 3, 4])
def test_refinement_independent_of_numbering_and_orientation(L):
    """Renumber the macro nodes and give every element a random rotation of its corner
    order: the refined operator must stay the same (shared edge and face nodes)."""
    m = read_sfem_mesh(FIXTURE)
    rng = np.random.default_rng(L)
    newid = rng.permutation(m.n_nodes)
    pts = np.empty_like(m.points)
    pts[:, newid] = m.points
    el = newid[m.elements]
    rots = _rotations()
    key = {tuple(c): k for k, c in enumerate(HEX8_CORNERS)}
    out = np.empty_like(el)
    for e in range(m.n_elements):
        R = rots[rng.integers(len(rots))]
        for k in range(8):
            src = (R @ (2 * HEX8_CORNERS[k] - 1) + 1) // 2
            out[k, e] = el[key[tuple(src)], e]
    bnd = {k: newid[v] for k, v in m.boundary_nodes.items()}
    hm = HexSSMesh(out, pts, L, boundary=bnd)
    _compare_with_structured(hm, L)


def test_write_read_roundtrip(tmp_path):
    m = read_sfem_mesh(FIXTURE)
    write_sfem_mesh(tmp_path / "copy", m)
    r = read_sfem_mesh(tmp_path / "copy")
    assert r.element_type == m.element_type
    assert np.array_equal(r.elements, m.elements) and np.array_equal(r.points, m.points)
    assert {k: list(v) for k, v in r.boundary_nodes.items()} == {k: list(v) for k, v in m.boundary_nodes.items()}
    meta = parse_meta((FIXTURE / "meta.yaml").read_text())
    assert parse_meta(format_meta(meta)) == meta
    assert meta["n_elements"] == 12 and meta["rpath"] is True
    assert meta["elements"][3] == {"i3": "i3.raw"}


def test_bad_meshes(tmp_path):
    m = read_sfem_mesh(FIXTURE)
    bad = SfemMesh("HEX8", m.elements.copy(), m.points)
    bad.elements[0, 0] = 99
    write_sfem_mesh(tmp_path / "bad", bad)
    with pytest.raises(ValueError, match="outside"):
        read_sfem_mesh(tmp_path / "bad")
    write_sfem_mesh(tmp_path / "tet", SfemMesh("TET4", m.elements[:4], m.points))
    with pytest.raises(ValueError, match="HEX8"):
        ssmesh_from_folder(tmp_path / "tet", 2)
    with pytest.raises(KeyError):
        HexSSMesh(m.elements, m.points, 2).boundary_nodes("left")


def test_read_wide_types_and_comments(tmp_path):
    """int64 ids and float64 coordinates named in the file names, comments and quoted
    values in meta.yaml, boundary files named without their folder."""
    m = read_sfem_mesh(FIXTURE)
    d = tmp_path / "wide"
    (d / "boundary_nodes").mkdir(parents=True)
    for v in range(8):
        m.elements[v].astype(np.int64).tofile(d / f"i{v}.int64.raw")
    for k, name in enumerate("xyz"):
        m.points[k].astype(np.float64).tofile(d / f"{name}.float64.raw")
    m.boundary_nodes["left"].astype(np.int64).tofile(d / "boundary_nodes" / "left.int64.raw")
    lines = ["# written by hand", "element_type: 'HEX8'  # quoted", f"n_elements: {m.n_elements}",
             f"n_points: {m.n_nodes}", "rpath: true", "elements:"]
    lines += [f"- i{v}: i{v}.int64.raw" for v in range(8)]
    lines += ["points:"] + [f"- {n}: {n}.float64.raw" for n in "xyz"]
    lines += ["boundary_nodes:", "- left: left.int64.raw"]
    (d / "meta.yaml").write_text("\n".join(lines) + "\n")
    r = read_sfem_mesh(d)
    assert r.element_type == "HEX8"
    assert np.array_equal(r.elements, m.elements) and np.array_equal(r.points, m.points)
    assert np.array_equal(r.boundary_nodes["left"], m.boundary_nodes["left"])
    hm = ssmesh_from_folder(d, 2)
    assert hm.n_nodes(2) == 7 * 5 * 5 and hm.boundary_nodes("left", 2).size == 5 * 5


@pytest.mark.parametrize("L", [2, 4])
def test_sshex8_to_hex8_micro_mesh(tmp_path, L):
    """The micro hex8 mesh of an (affine) sshex8 level carries the same Laplacian, and
    survives a write / read as a reference mesh folder."""
    from sfem_gb300.meshio import sshex8_to_hex8

    m = SSMesh(3, 2, 2, L, box=((0, 2), (0, 1), (0, 1)))
    el = m.elements(L)
    micro = sshex8_to_hex8(el, L)
    assert micro.shape == (8, m.n_elements * L ** 3)
    write_sfem_mesh(tmp_path / "micro", SfemMesh("HEX8", micro, m.points))
    r = read_sfem_mesh(tmp_path / "micro")
    assert np.array_equal(r.elements, micro)
    x = np.random.default_rng(L).standard_normal(m.n_nodes(L))
    fff_macro = O.fff_fill(el[m.macro_corner_lidx(L)], m.points)
    y_ss = O.sshex8_laplacian_apply(L, el, fff_macro, x)
    # same operator, one metric per micro element: the macro FFF / L (exact in float for
    # L = 2, 4) gives the hex8 apply the sshex8 apply's coefficients, so they agree to
    # summation order (a node-ordering or sign error would show at O(1))
    fff_micro = np.repeat(fff_macro / np.float32(L), L ** 3, axis=0)
    y_h8 = O.hex8_laplacian_apply(r.elements, fff_micro, x)
    assert np.abs(y_h8 - y_ss).max() <= 1e-12 * np.abs(y_ss).max()
    # and the metric of the micro elements' own coordinates agrees to float rounding
    y_geo = O.hex8_laplacian_apply(r.elements, O.fff_fill(r.elements, r.points), x)
    assert np.abs(y_geo - y_ss).max() <= 1e-6 * np.abs(y_ss).max()
