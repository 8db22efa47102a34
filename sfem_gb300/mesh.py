"""Semi-structured hex8 (sshex8) mesh hierarchies on a box.

The reference delegates mesh construction to its ``smesh`` submodule
(``Mesh::create_hex8_cube``, ``to_semistructured``, ``derefinement_levels``),
called from ``frontend/sfem_API.hpp:409-584`` and
``algebra/mg/sfem_GeometricMultigrid.cpp:25``.  That submodule is not part of
the reference snapshot, so this module restates what the operator path needs
from it, with the reference's array conventions:

* connectivity is SoA ``elements[lidx][e]`` (int32), with the sshex8 local
  index ``lidx = z*(L+1)^2 + y*(L+1) + x`` (``operators/sshex8/sshex8.hpp:18-24``);
* plain hex8 connectivity uses the standard corner order
  (x,y,z),(x+1,y,z),(x+1,y+1,z),(x,y+1,z) then the same at z+1
  (``operators/sshex8/sshex8_laplacian.cpp:47-57``);
* points are SoA float32 ``points[d][node]``.

Node numbering is *nested*: the nodes of every coarser level of the
derefinement hierarchy come first, so a level-``l`` vector is a prefix of the
finest vector.  This is what the reference's hierarchical transfer needs
(``sshex8_hierarchical_prolongation`` reads the coarse hex8 vector through the
sshex8 corner indices, ``operators/sshex8/sshex8_interpolate.cpp:129-237``).
Within one level group nodes are ordered lexicographically (x fastest).

Macro element ``e = a + nx*(b + ny*c)`` for macro position ``(a, b, c)``.
"""

from __future__ import annotations

import numpy as np


def derefinement_levels(L: int) -> list[int]:
    """Levels of the sshex8 multigrid hierarchy, finest first.

    Halve while even, and always end at the plain hex8 level 1
    (4 -> [4, 2, 1]; 3 -> [3, 1]; 6 -> [6, 3, 1]).
    """
    if L < 1:
        raise ValueError("level must be >= 1")
    levels = [L]
    l = L
    while l > 1 and l % 2 == 0:
        l //= 2
        levels.append(l)
    if levels[-1] != 1:
        levels.append(1)
    return levels


def sshex8_nxe(L: int) -> int:
    return (L + 1) ** 3


def sshex8_lidx(L: int, x, y, z):
    return z * (L + 1) * (L + 1) + y * (L + 1) + x


# hex8 corner k -> (x, y, z) offset in the standard order
HEX8_CORNERS = np.array(
    [[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0], [0, 0, 1], [1, 0, 1], [1, 1, 1], [0, 1, 1]],
    dtype=np.int64,
)


def perturbed_macro_points(nx, ny, nz, box=((0.0, 1.0), (0.0, 1.0), (0.0, 1.0)), perturb=0.0, seed=0) -> np.ndarray:
    """Macro node coordinates ``[3, nz+1, ny+1, nx+1]`` (float64) of a box: a uniform
    grid whose interior nodes move by U(-perturb, perturb)*h per coordinate (seeded)."""
    (x0, x1), (y0, y1), (z0, z1) = box
    hx, hy, hz = (x1 - x0) / nx, (y1 - y0) / ny, (z1 - z0) / nz
    X = x0 + hx * np.arange(nx + 1, dtype=np.float64)
    Y = y0 + hy * np.arange(ny + 1, dtype=np.float64)
    Z = z0 + hz * np.arange(nz + 1, dtype=np.float64)
    MZ, MY, MX = np.meshgrid(Z, Y, X, indexing="ij")
    macro = np.stack([MX, MY, MZ])
    if perturb > 0:
        rng = np.random.default_rng(seed)
        noise = rng.uniform(-perturb, perturb, size=macro.shape)
        noise[0] *= hx
        noise[1] *= hy
        noise[2] *= hz
        interior = np.zeros(macro.shape[1:], dtype=bool)
        interior[1:-1, 1:-1, 1:-1] = True
        macro = macro + noise * interior[None]
    return macro


class SSMesh:
    """A box meshed by ``nx*ny*nz`` macro hex8 elements refined at level ``L``.

    ``perturb`` moves every interior *macro* node by U(-perturb, perturb)*h in
    each coordinate (seeded).  Micro nodes are placed by trilinear
    interpolation of their macro element's corners, as a semi-structured
    refinement of the macro mesh does.  The affine sshex8 kernels only read
    the macro corners (geometry is one metric per macro element,
    ``operators/sshex8/sshex8_laplacian.cpp:698-769``).
    """

    def __init__(self, nx, ny, nz, L, box=((0.0, 1.0), (0.0, 1.0), (0.0, 1.0)), perturb=0.0, seed=0):
        self.nx, self.ny, self.nz, self.L = int(nx), int(ny), int(nz), int(L)
        self.box = tuple(tuple(float(v) for v in b) for b in box)
        self.levels = derefinement_levels(self.L)
        self.perturb = float(perturb)
        self.seed = int(seed)
        self.n_elements = self.nx * self.ny * self.nz
        self._build_numbering()
        self._build_points()
        self._elements = {}

    # ------------------------------------------------------------------ numbering
    def grid_shape(self, l=None):
        l = self.L if l is None else l
        return (l * self.nx + 1, l * self.ny + 1, l * self.nz + 1)

    def n_nodes(self, l=None) -> int:
        gx, gy, gz = self.grid_shape(l)
        return gx * gy * gz

    def _build_numbering(self):
        L = self.L
        gx, gy, gz = self.grid_shape()
        i = np.arange(gx, dtype=np.int64)
        j = np.arange(gy, dtype=np.int64)
        k = np.arange(gz, dtype=np.int64)
        # group of a fine position: index of the coarsest level that contains it
        levels_coarse_first = sorted(self.levels)
        group = np.full((gz, gy, gx), len(levels_coarse_first), dtype=np.int8)
        for g, l in reversed(list(enumerate(levels_coarse_first))):
            s = L // l
            mask = (k[:, None, None] % s == 0) & (j[None, :, None] % s == 0) & (i[None, None, :] % s == 0)
            group[mask] = g
        flat_group = group.reshape(-1)
        order = np.argsort(flat_group, kind="stable")
        node_of_flat = np.empty(order.size, dtype=np.int64)
        node_of_flat[order] = np.arange(order.size, dtype=np.int64)
        self._node_of_flat = node_of_flat
        self._flat_of_node = order
        # sanity: each level is a prefix
        for l in self.levels:
            assert int(np.count_nonzero(flat_group <= levels_coarse_first.index(l))) == self.n_nodes(l)

    def node_id(self, i, j, k):
        """Node id of fine-grid position (i, j, k) (arrays allowed)."""
        gx, gy, _ = self.grid_shape()
        return self._node_of_flat[np.asarray(i) + gx * (np.asarray(j) + gy * np.asarray(k))]

    def fine_position(self, node):
        gx, gy, _ = self.grid_shape()
        f = self._flat_of_node[np.asarray(node)]
        return f % gx, (f // gx) % gy, f // (gx * gy)

    # ------------------------------------------------------------------ elements
    def macro_positions(self):
        e = np.arange(self.n_elements, dtype=np.int64)
        a = e % self.nx
        b = (e // self.nx) % self.ny
        c = e // (self.nx * self.ny)
        return a, b, c

    def elements(self, l=None) -> np.ndarray:
        """sshex8 connectivity at level ``l``: int32 array ``[(l+1)^3, E]``."""
        l = self.L if l is None else int(l)
        if l not in self.levels:
            raise ValueError(f"level {l} not in hierarchy {self.levels}")
        if l in self._elements:
            return self._elements[l]
        s = self.L // l
        a, b, c = self.macro_positions()
        n = l + 1
        zi, yi, xi = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
        xi, yi, zi = xi.reshape(-1), yi.reshape(-1), zi.reshape(-1)  # lidx order
        I = a[None, :] * self.L + xi[:, None] * s
        J = b[None, :] * self.L + yi[:, None] * s
        K = c[None, :] * self.L + zi[:, None] * s
        el = self.node_id(I, J, K).astype(np.int32)
        el = np.ascontiguousarray(el)
        self._elements[l] = el
        return el

    def hex8_elements(self) -> np.ndarray:
        """Plain hex8 connectivity of the macro mesh (standard corner order), int32 ``[8, E]``."""
        el1 = self.elements(1)
        lid = [sshex8_lidx(1, *HEX8_CORNERS[k]) for k in range(8)]
        return np.ascontiguousarray(el1[lid])

    def macro_corner_lidx(self, l=None):
        """lidx (at level l) of the 8 macro corners in standard hex8 order."""
        l = self.L if l is None else l
        return [sshex8_lidx(l, *(HEX8_CORNERS[k] * l)) for k in range(8)]

    # ------------------------------------------------------------------ geometry
    def _build_points(self):
        nx, ny, nz, L = self.nx, self.ny, self.nz, self.L
        macro = perturbed_macro_points(nx, ny, nz, self.box, self.perturb, self.seed)
        self.macro_points = macro.astype(np.float32)
        # fine nodes: trilinear interpolation inside the owning macro cell
        gx, gy, gz = self.grid_shape()
        i = np.arange(gx)
        j = np.arange(gy)
        k = np.arange(gz)
        ai = np.minimum(i // L, nx - 1)
        bj = np.minimum(j // L, ny - 1)
        ck = np.minimum(k // L, nz - 1)
        ti = (i - ai * L) / L
        tj = (j - bj * L) / L
        tk = (k - ck * L) / L
        m = macro.astype(np.float32).astype(np.float64)
        pts = np.zeros((3, gz, gy, gx), dtype=np.float64)
        for dz in (0, 1):
            wz = (tk if dz else 1 - tk)[:, None, None]
            for dy in (0, 1):
                wy = (tj if dy else 1 - tj)[None, :, None]
                for dx in (0, 1):
                    wx = (ti if dx else 1 - ti)[None, None, :]
                    corner = m[:, (ck + dz)[:, None, None], (bj + dy)[None, :, None], (ai + dx)[None, None, :]]
                    pts += corner * (wz * wy * wx)[None]
        # at macro nodes use the exact (float32) macro coordinates
        flat = pts.reshape(3, -1)
        points = np.empty((3, flat.shape[1]), dtype=np.float32)
        points[:, self._node_of_flat] = flat.astype(np.float32)
        self.points = points

    # ------------------------------------------------------------------ boundary
    def boundary_nodes(self, face: str, l=None) -> np.ndarray:
        """Sorted node ids (< n_nodes(l)) on a box face: 'x0','x1','y0','y1','z0','z1'."""
        l = self.L if l is None else l
        s = self.L // l
        gx, gy, gz = self.grid_shape(l)
        i = np.arange(gx) * s
        j = np.arange(gy) * s
        k = np.arange(gz) * s
        Lx, Ly, Lz = self.grid_shape()
        axis, side = face[0], face[1]
        if axis == "x":
            K, J = np.meshgrid(k, j, indexing="ij")
            I = np.full_like(K, 0 if side == "0" else Lx - 1)
        elif axis == "y":
            K, I = np.meshgrid(k, i, indexing="ij")
            J = np.full_like(K, 0 if side == "0" else Ly - 1)
        elif axis == "z":
            J, I = np.meshgrid(j, i, indexing="ij")
            K = np.full_like(J, 0 if side == "0" else Lz - 1)
        else:
            raise ValueError(face)
        ids = self.node_id(I.reshape(-1), J.reshape(-1), K.reshape(-1))
        return np.unique(ids).astype(np.int32)

    def all_boundary_nodes(self, l=None) -> np.ndarray:
        return np.unique(np.concatenate([self.boundary_nodes(f, l) for f in ("x0", "x1", "y0", "y1", "z0", "z1")])).astype(np.int32)


def hex8_cube(n: int, perturb=0.0, seed=0) -> SSMesh:
    """Structured hex8 mesh of the unit cube with ``n^3`` elements (level 1)."""
    return SSMesh(n, n, n, 1, perturb=perturb, seed=seed)


def upper_crs_graph(elements: np.ndarray, n_nodes: int):
    """Strict-upper node-to-node CRS graph (sorted columns > row) of an element mesh.

    ``elements`` is ``[nodes_per_element, E]``.  This is the graph the
    symmetric CRS / BSR formats and their assembly kernels use (the reference
    builds it with smesh's ``create_node_to_node_graph``).
    """
    nv, E = elements.shape
    el = elements.astype(np.int64)
    rows = np.repeat(el, nv, axis=0).reshape(nv, nv, E)
    cols = np.tile(el, (nv, 1)).reshape(nv, nv, E)
    r, c = rows.reshape(-1), cols.reshape(-1)
    keep = c > r
    key = np.unique(r[keep] * n_nodes + c[keep])
    r, c = key // n_nodes, key % n_nodes
    rowptr = np.zeros(n_nodes + 1, dtype=np.int64)
    np.add.at(rowptr, r + 1, 1)
    rowptr = np.cumsum(rowptr).astype(np.int32)
    return rowptr, c.astype(np.int32)


def full_crs_graph(elements: np.ndarray, n_nodes: int):
    """Node-to-node CRS graph with both triangles and the diagonal (sorted columns): the
    pattern of the full CRS and BSR assembly (the reference's node-to-node graph)."""
    nv, E = elements.shape
    el = elements.astype(np.int64)
    r = np.repeat(el, nv, axis=0).reshape(-1)
    c = np.tile(el, (nv, 1)).reshape(-1)
    key = np.unique(r * n_nodes + c)
    r, c = key // n_nodes, key % n_nodes
    rowptr = np.zeros(n_nodes + 1, dtype=np.int64)
    np.add.at(rowptr, r + 1, 1)
    rowptr = np.cumsum(rowptr).astype(np.int32)
    return rowptr, c.astype(np.int32)


def _coarse_axis(n: int) -> np.ndarray:
    """Finer-grid indices kept on a 2x coarser axis of n elements: the even ones,
    plus the last index when n is odd (the last coarse element then spans one
    finer element)."""
    idx = list(range(0, n + 1, 2))
    if n % 2:
        idx.append(n)
    return np.asarray(idx, dtype=np.int64)


def _interp_1d(n: int, kept: np.ndarray) -> np.ndarray:
    """Dense (n+1) x len(kept) linear interpolation from the kept nodes to all nodes."""
    P = np.zeros((n + 1, kept.size))
    for i in range(n + 1):
        b = int(np.searchsorted(kept, i))
        if kept[b] == i:
            P[i, b] = 1.0
        else:
            a = b - 1
            t = (i - kept[a]) / (kept[b] - kept[a])
            P[i, a] = 1.0 - t
            P[i, b] = t
    return P


class CoarseHex8Level:
    """A plain hex8 level made by coarsening a structured hex8 grid 2x in every direction.

    The reference's sshex8 hierarchy ends at the hex8 macro mesh, whose solve it
    hands to a coarse solver (``algebra/mg/sfem_GeometricMultigrid.cpp``).  On box
    meshes the macro grid is itself structured, so geometric multigrid can go on
    below it: the finer grid's nodes at even positions (and the last one of an odd
    axis) form the coarse grid, which is nested in the finer one and keeps its
    geometry.  The transfer is the trilinear nested interpolation P (CSR, finer
    rows) and its transpose R.

    ``fine_points``: float32 ``[3, gz, gy, gx]`` coordinates of the finer grid
    nodes; ``fine_ids``: int ``[gz, gy, gx]`` their ids in the finer vector.
    Coarse nodes are numbered lexicographically (x fastest), coarse elements
    ``e = a + cx*(b + cy*c)``.
    """

    def __init__(self, fine_points: np.ndarray, fine_ids: np.ndarray):
        from scipy import sparse

        gz, gy, gx = fine_ids.shape
        kx, ky, kz = _coarse_axis(gx - 1), _coarse_axis(gy - 1), _coarse_axis(gz - 1)
        cx, cy, cz = kx.size - 1, ky.size - 1, kz.size - 1
        self.shape = (cx, cy, cz)
        self.n_elements = cx * cy * cz
        self.n_nodes = (cx + 1) * (cy + 1) * (cz + 1)
        self.ids = np.arange(self.n_nodes, dtype=np.int64).reshape(cz + 1, cy + 1, cx + 1)
        self.points_grid = np.ascontiguousarray(fine_points[:, kz][:, :, ky][:, :, :, kx]).astype(np.float32)
        self.points = np.ascontiguousarray(self.points_grid.reshape(3, -1))
        e = np.arange(self.n_elements, dtype=np.int64)
        a, b, c = e % cx, (e // cx) % cy, e // (cx * cy)
        self.hex8 = np.ascontiguousarray(np.stack(
            [self.ids[c + dz, b + dy, a + dx] for dx, dy, dz in HEX8_CORNERS]).astype(np.int32))
        # P: finer (lexicographic, then renumbered by fine_ids) x coarse (lexicographic)
        Px = sparse.csr_matrix(_interp_1d(gx - 1, kx))
        Py = sparse.csr_matrix(_interp_1d(gy - 1, ky))
        Pz = sparse.csr_matrix(_interp_1d(gz - 1, kz))
        P = sparse.kron(Pz, sparse.kron(Py, Px)).tocsr()
        perm = np.empty(fine_ids.size, dtype=np.int64)
        perm[fine_ids.reshape(-1)] = np.arange(fine_ids.size)  # fine id -> lexicographic row
        P = P[perm].tocsr()
        P.sort_indices()
        self.n_fine_nodes = int(fine_ids.size)
        self.P = (P.indptr.astype(np.int32), P.indices.astype(np.int32), P.data.astype(np.float64))
        R = P.T.tocsr()
        R.sort_indices()
        self.R = (R.indptr.astype(np.int32), R.indices.astype(np.int32), R.data.astype(np.float64))

    def can_coarsen(self) -> bool:
        return all(n >= 2 for n in self.shape)

    def coarser(self) -> "CoarseHex8Level":
        return CoarseHex8Level(self.points_grid, self.ids)

    def boundary_nodes(self, face: str) -> np.ndarray:
        axis, side = face[0], face[1]
        idx = 0 if side == "0" else -1
        sl = {"x": (slice(None), slice(None), idx), "y": (slice(None), idx, slice(None)),
              "z": (idx, slice(None), slice(None))}[axis]
        return np.unique(self.ids[sl].reshape(-1)).astype(np.int32)


def macro_level_grid(mesh: SSMesh):
    """(points ``[3, nz+1, ny+1, nx+1]``, ids ``[nz+1, ny+1, nx+1]``) of the level-1 (macro) grid of ``mesh``."""
    L = mesh.L
    K, J, I = np.meshgrid(np.arange(mesh.nz + 1), np.arange(mesh.ny + 1), np.arange(mesh.nx + 1), indexing="ij")
    ids = mesh.node_id(I * L, J * L, K * L)
    return mesh.macro_points, ids


def coarse_shape(shape):
    return tuple((n + 1) // 2 for n in shape)


def macro_coarse_levels(mesh: SSMesh, min_nodes: int = 64) -> list:
    """Coarse hex8 levels below the macro mesh, finest first: 2x coarsening (odd axes
    keep a thin last element) while every axis has at least 2 elements and the
    next level keeps at least ``min_nodes`` nodes."""
    pts, ids = macro_level_grid(mesh)
    out = []
    shape = (mesh.nx, mesh.ny, mesh.nz)
    while all(n >= 2 for n in shape):
        cs = coarse_shape(shape)
        if int(np.prod([n + 1 for n in cs])) < min_nodes:
            break
        nxt = CoarseHex8Level(pts, ids) if not out else out[-1].coarser()
        out.append(nxt)
        shape = nxt.shape
    return out


def coarsen_coefficient(k: np.ndarray, shape) -> np.ndarray:
    """Per-element coefficient ``k[z, y, x]`` of a grid, averaged onto its 2x coarser grid
    of ``shape`` (z, y, x): the mean of the (up to 2x2x2) children of each coarse element
    (an odd axis ends in a thin element with one child layer)."""
    out = np.asarray(k, dtype=np.float64)
    for axis, n in enumerate(shape):
        m = out.shape[axis]
        parts = [np.take(out, list(range(2 * i, min(2 * i + 2, m))), axis=axis).mean(axis=axis, keepdims=True)
                 for i in range(n)]
        out = np.concatenate(parts, axis=axis)
    return out
