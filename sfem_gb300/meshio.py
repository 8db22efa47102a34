"""SFEM on-disk meshes and semi-structured refinement of any conforming hex8 mesh.

The reference stores a mesh as a folder (written by
``python/sfem/mesh/box_mesh.py:781-884``, read by smesh's
``Mesh::create_from_file`` in ``drivers/mgsolve.cpp:53``): ``meta.yaml`` with
``element_type``, ``n_elements``, ``n_points``, ``elements: [- i0: i0.raw, ...]``,
``points: [- x: x.raw, ...]`` and ``boundary_nodes: [- left: left.int32.raw, ...]``;
one raw little-endian file per connectivity row (int32 ``idx_t``), per
coordinate (float32 ``geom_t``) and per boundary node set (int32).  Paths are
relative to the folder (``rpath: true``).  :func:`read_sfem_mesh` and
:func:`write_sfem_mesh` handle that format (meta.yaml through a small parser of
the block-style subset the reference writes: PyYAML is not a dependency here).

:class:`HexSSMesh` refines an arbitrary conforming hex8 mesh (any node
numbering, any corner orientation per element) to a semi-structured sshex8
mesh of level ``L``, the role of smesh's ``to_semistructured``: nodes on a
macro edge or face are shared by every element that contains it, through a
canonical parameterisation of the entity (edges from the end with the smaller
macro id; faces from the corner with the smallest macro id, first axis towards
its smaller neighbour).  The numbering is nested like
:class:`sfem_gb300.mesh.SSMesh`: the nodes of every coarser derefinement level
come first, so the class plugs into :class:`sfem_gb300.operators.SSMeshDevice`
and :class:`sfem_gb300.solvers.Hierarchy` (without ``coarsen_macro``, which
needs a structured macro grid).
"""

from __future__ import annotations

import re
from pathlib import Path

import numpy as np

from .mesh import HEX8_CORNERS, derefinement_levels, sshex8_lidx

_DTYPES = {"int16": np.int16, "int32": np.int32, "int64": np.int64, "float32": np.float32, "float64": np.float64}


# ---------------------------------------------------------------------- meta.yaml
def _scalar(v: str):
    v = v.strip()
    if len(v) >= 2 and v[0] == v[-1] and v[0] in "'\"":
        return v[1:-1]
    if v in ("true", "True"):
        return True
    if v in ("false", "False"):
        return False
    try:
        return int(v)
    except ValueError:
        pass
    try:
        return float(v)
    except ValueError:
        return v


def parse_meta(text: str) -> dict:
    """Block-style YAML subset of the reference's meta files: ``key: scalar`` and
    ``key:`` followed by ``- name: value`` items (lists of one-entry maps)."""
    meta: dict = {}
    current = None
    for raw in text.splitlines():
        line = raw.split("#", 1)[0].rstrip() if not raw.lstrip().startswith("#") else ""
        if not line.strip():
            continue
        s = line.strip()
        if s.startswith("- "):
            if current is None:
                raise ValueError(f"meta.yaml: list item outside a list: {raw!r}")
            item = s[2:]
            if ":" in item:
                k, v = item.split(":", 1)
                meta[current].append({k.strip(): _scalar(v)})
            else:
                meta[current].append(_scalar(item))
            continue
        if line[0] in " \t" and current is not None and ":" in s:
            # continuation of the last list item's map
            k, v = s.split(":", 1)
            meta[current][-1][k.strip()] = _scalar(v)
            continue
        if ":" not in s:
            raise ValueError(f"meta.yaml: cannot parse {raw!r}")
        k, v = s.split(":", 1)
        k = k.strip()
        if v.strip() == "":
            meta[k] = []
            current = k
        elif v.strip() == "[]":
            meta[k] = []
            current = None
        else:
            meta[k] = _scalar(v)
            current = None
    return meta


def format_meta(meta: dict) -> str:
    """meta.yaml text in the block style the reference writes (keys sorted, as PyYAML's dump)."""
    out = ["# SFEM mesh meta file"]
    for k in sorted(meta):
        v = meta[k]
        if isinstance(v, list):
            out.append(f"{k}:")
            for item in v:
                if isinstance(item, dict):
                    (ik, iv), = item.items()
                    out.append(f"- {ik}: {_fmt(iv)}")
                else:
                    out.append(f"- {_fmt(item)}")
        else:
            out.append(f"{k}: {_fmt(v)}")
    return "\n".join(out) + "\n"


def _fmt(v) -> str:
    if isinstance(v, bool):
        return "true" if v else "false"
    return str(v)


def _raw_dtype(name: str, default):
    for tok in re.split(r"[._]", name):
        if tok in _DTYPES:
            return _DTYPES[tok]
    return default


# ---------------------------------------------------------------------- folders
class SfemMesh:
    """A mesh folder in memory: ``elements[v][e]`` (int32), ``points[d][node]``
    (float32) and named boundary node sets (int32)."""

    def __init__(self, element_type: str, elements: np.ndarray, points: np.ndarray, boundary_nodes=None):
        self.element_type = element_type
        self.elements = np.ascontiguousarray(elements, dtype=np.int32)
        self.points = np.ascontiguousarray(points, dtype=np.float32)
        self.boundary_nodes = {k: np.asarray(v, dtype=np.int32) for k, v in (boundary_nodes or {}).items()}

    @property
    def n_elements(self) -> int:
        return int(self.elements.shape[1])

    @property
    def n_nodes(self) -> int:
        return int(self.points.shape[1])


def read_sfem_mesh(folder) -> SfemMesh:
    """Read a reference mesh folder (meta.yaml + raw arrays)."""
    folder = Path(folder)
    meta = parse_meta((folder / "meta.yaml").read_text())

    def path(name):
        p = Path(str(name))
        return p if p.is_absolute() else folder / p

    def entries(key):
        items = meta.get(key) or []
        return [next(iter(it.items())) for it in items]

    etype = str(meta.get("element_type", "HEX8"))
    rows = [np.fromfile(path(f), dtype=_raw_dtype(str(f), np.int32)) for _, f in entries("elements")]
    pts = [np.fromfile(path(f), dtype=_raw_dtype(str(f), np.float32)) for _, f in entries("points")]
    if not rows or not pts:
        raise ValueError(f"{folder}: meta.yaml lists no elements or points")
    elements = np.stack(rows).astype(np.int32)
    points = np.stack(pts).astype(np.float32)
    if "n_elements" in meta and elements.shape[1] != int(meta["n_elements"]):
        raise ValueError(f"{folder}: {elements.shape[1]} elements on disk, meta says {meta['n_elements']}")
    if "n_points" in meta and points.shape[1] != int(meta["n_points"]):
        raise ValueError(f"{folder}: {points.shape[1]} points on disk, meta says {meta['n_points']}")
    if elements.size and (elements.min() < 0 or elements.max() >= points.shape[1]):
        raise ValueError(f"{folder}: element node ids outside [0, {points.shape[1]})")
    bnd = {}
    for name, f in entries("boundary_nodes"):
        p = path(f)
        if not p.exists():
            p = folder / "boundary_nodes" / str(f)
        bnd[name] = np.fromfile(p, dtype=_raw_dtype(str(f), np.int32)).astype(np.int32)
    return SfemMesh(etype, elements, points, bnd)


def write_sfem_mesh(folder, mesh: SfemMesh) -> None:
    """Write ``mesh`` as a reference mesh folder."""
    folder = Path(folder)
    folder.mkdir(parents=True, exist_ok=True)
    meta = {"element_type": mesh.element_type, "spatial_dimension": int(mesh.points.shape[0]), "rpath": True,
            "n_points": mesh.n_nodes, "n_elements": mesh.n_elements, "elem_num_nodes": int(mesh.elements.shape[0])}
    meta["points"] = []
    for d, name in enumerate("xyz"[: mesh.points.shape[0]]):
        mesh.points[d].astype(np.float32).tofile(folder / f"{name}.raw")
        meta["points"].append({name: f"{name}.raw"})
    meta["elements"] = []
    for v in range(mesh.elements.shape[0]):
        mesh.elements[v].astype(np.int32).tofile(folder / f"i{v}.raw")
        meta["elements"].append({f"i{v}": f"i{v}.raw"})
    if mesh.boundary_nodes:
        (folder / "boundary_nodes").mkdir(exist_ok=True)
        meta["boundary_nodes"] = []
        for k, v in mesh.boundary_nodes.items():
            np.asarray(v, dtype=np.int32).tofile(folder / "boundary_nodes" / f"{k}.int32.raw")
            meta["boundary_nodes"].append({k: f"boundary_nodes/{k}.int32.raw"})
    (folder / "meta.yaml").write_text(format_meta(meta))


# ---------------------------------------------------------------------- refinement
# the 12 edges of the reference hex (corner pairs along x, y, z) and the 6 faces as
# (fixed axis, side, the two in-face axes a < b)
_EDGES = [(a, b) for a in range(8) for b in range(a + 1, 8)
          if int(np.abs(HEX8_CORNERS[a] - HEX8_CORNERS[b]).sum()) == 1]
_FACES = [(d, s) for d in range(3) for s in (0, 1)]


def _corner_of(offset) -> int:
    return int(np.flatnonzero((HEX8_CORNERS == np.asarray(offset)).all(axis=1))[0])


class HexSSMesh:
    """Level-``L`` semi-structured refinement of a conforming hex8 mesh.

    ``hex_elements``: ``[8, E]`` corner ids in the standard hex8 order;
    ``points``: ``[3, N]`` float32; ``boundary``: named macro node sets (a set's
    refinement = every micro node on a boundary face whose four corners are in
    the set).  Same interface as :class:`sfem_gb300.mesh.SSMesh` for the device
    path: ``L``, ``levels``, ``n_elements``, ``n_nodes(l)``, ``elements(l)``,
    ``hex8_elements()``, ``macro_corner_lidx(l)``, ``points``,
    ``boundary_nodes(name, l)``."""

    def __init__(self, hex_elements, points, L: int, boundary=None):
        hx = np.asarray(hex_elements, dtype=np.int64)
        if hx.ndim != 2 or hx.shape[0] != 8:
            raise ValueError("hex_elements must be [8, E]")
        if L < 1:
            raise ValueError("level must be >= 1")
        self.L = int(L)
        self.levels = derefinement_levels(self.L)
        self.n_elements = int(hx.shape[1])
        self._boundary = {k: np.asarray(v, dtype=np.int64) for k, v in (boundary or {}).items()}
        self._hex = hx
        self._macro_points = np.asarray(points, dtype=np.float32)
        self._build()
        self._elements = {}

    # -------------------------------------------------------------- numbering
    def _build(self):
        L, E, hx = self.L, self.n_elements, self._hex
        n1 = L + 1
        # lattice of one element at level L
        zz, yy, xx = np.meshgrid(np.arange(n1), np.arange(n1), np.arange(n1), indexing="ij")
        lat = np.stack([xx.reshape(-1), yy.reshape(-1), zz.reshape(-1)])  # [3, nxe] in lidx order
        nxe = lat.shape[1]
        onb = (lat == 0) | (lat == L)
        nb = onb.sum(axis=0)
        prov = np.full((nxe, E), -1, dtype=np.int64)  # provisional node id per (lattice point, element)
        canon = np.zeros((3, nxe, E), dtype=np.int64)  # canonical entity coordinates (for the level groups)
        # vertices: the referenced macro nodes, compacted
        verts, vmap = np.unique(hx, return_inverse=True)
        vmap = vmap.reshape(hx.shape)
        self._vertex_ids = verts
        base = verts.size
        for v in np.flatnonzero(nb == 3):
            c = _corner_of(lat[:, v] // L)
            prov[v] = vmap[c]
        # faces: key = sorted corner ids; canonical origin = smallest corner id
        fkeys, finfo = [], []
        for d, side in _FACES:
            a, b = [ax for ax in range(3) if ax != d]
            cs = []
            for (ua, vb) in ((0, 0), (1, 0), (1, 1), (0, 1)):  # cyclic
                off = np.zeros(3, dtype=int)
                off[d], off[a], off[b] = side, ua, vb
                cs.append(_corner_of(off))
            ids = hx[cs]  # [4, E] cyclic
            fkeys.append(np.sort(ids, axis=0))
            finfo.append((d, side, a, b, ids))
        fk = np.stack(fkeys, axis=1)  # [4, 6, E]
        flat = fk.reshape(4, -1).T
        ufaces, fid, fcount = np.unique(flat, axis=0, return_inverse=True, return_counts=True)
        fid = fid.reshape(6, E)
        self._face_multiplicity = fcount[fid]  # [6, E]
        self._face_keys = ufaces
        self._face_id = fid
        # edges: key (min, max) macro id, parameter from the smaller id
        if L > 1:
            ea = np.array([a for a, _ in _EDGES])
            eb = np.array([b for _, b in _EDGES])
            ida, idb = hx[ea], hx[eb]  # [12, E]
            lo, hi = np.minimum(ida, idb), np.maximum(ida, idb)
            keys = lo * (hx.max() + 1) + hi
            ukeys, eid = np.unique(keys.reshape(-1), return_inverse=True)
            eid = eid.reshape(keys.shape)
            for k, (a, b) in enumerate(_EDGES):
                d = int(np.flatnonzero(HEX8_CORNERS[a] != HEX8_CORNERS[b])[0])
                fixed = HEX8_CORNERS[a] * L
                for t in range(1, L):  # lattice coordinate along the edge
                    p = fixed.copy()
                    p[d] = t
                    v = sshex8_lidx(L, *p)
                    ta = t if HEX8_CORNERS[a, d] == 0 else L - t  # distance from corner a
                    s = np.where(ida[k] < idb[k], ta, L - ta)
                    prov[v] = base + eid[k] * (L - 1) + (s - 1)
                    canon[0, v] = s
            base += ukeys.size * (L - 1)
            for f, (d, side, a, b, ids) in enumerate(finfo):
                # cyclic corner j sits at in-face (u, v) = cyc[j] * L
                cyc = np.array([[0, 0], [1, 0], [1, 1], [0, 1]])
                j0 = np.argmin(ids, axis=0)  # origin corner (cyclic index)
                jn = (j0 + 1) % 4
                jp = (j0 + 3) % 4
                cols = np.arange(E)
                nxt_smaller = ids[jn, cols] < ids[jp, cols]
                j1 = np.where(nxt_smaller, jn, jp)  # first canonical axis towards this corner
                o = cyc[j0] * L  # [E, 2]
                dir1 = cyc[j1] - cyc[j0]  # unit step of the first canonical axis in (u, v)
                for u in range(1, L):
                    for w in range(1, L):
                        p = np.zeros(3, dtype=int)
                        p[d], p[a], p[b] = side * L, u, w
                        v = sshex8_lidx(L, *p)
                        du, dw = u - o[:, 0], w - o[:, 1]
                        along_u = dir1[:, 0] != 0
                        c1 = np.where(along_u, np.abs(du), np.abs(dw))
                        c2 = np.where(along_u, np.abs(dw), np.abs(du))
                        prov[v] = base + fid[f] * (L - 1) ** 2 + (c1 - 1) + (L - 1) * (c2 - 1)
                        canon[0, v], canon[1, v] = c1, c2
            base += ufaces.shape[0] * (L - 1) ** 2
            # interior
            inner = np.flatnonzero(nb == 0)
            for v in inner:
                x, y, z = lat[:, v]
                prov[v] = base + np.arange(E) * (L - 1) ** 3 + (x - 1) + (L - 1) * ((y - 1) + (L - 1) * (z - 1))
                canon[:, v] = lat[:, v][:, None]
            base += E * (L - 1) ** 3
        assert (prov >= 0).all()
        n_prov = base
        # nested groups: index (coarse first) of the coarsest level containing the node
        coarse_first = sorted(self.levels)
        group_pt = np.full((nxe, E), len(coarse_first), dtype=np.int64)
        for g in reversed(range(len(coarse_first))):
            st = L // coarse_first[g]
            ok = ((canon % st) == 0).all(axis=0)
            group_pt[ok] = g
        group = np.full(n_prov, -1, dtype=np.int64)
        group[prov.reshape(-1)] = group_pt.reshape(-1)
        assert (group >= 0).all()
        order = np.argsort(group, kind="stable")
        new_of_prov = np.empty(n_prov, dtype=np.int64)
        new_of_prov[order] = np.arange(n_prov)
        self._fine = new_of_prov[prov]  # [nxe, E] final ids at level L
        self._n_nodes = {l: int(np.count_nonzero(group <= coarse_first.index(l))) for l in self.levels}
        # points: trilinear map of each element at its lattice points (exact corners at vertices)
        P = self._macro_points.astype(np.float64)
        t = lat / float(L)
        pts = np.zeros((3, n_prov), dtype=np.float64)
        W = np.ones((8, nxe))
        for c in range(8):
            for d in range(3):
                W[c] *= t[d] if HEX8_CORNERS[c, d] else 1.0 - t[d]
        for d in range(3):
            val = np.einsum("cv,ce->ve", W, P[d][hx])
            pts[d, prov.reshape(-1)] = val.reshape(-1)
        pts[:, np.arange(verts.size)] = P[:, verts]
        out = np.empty((3, n_prov), dtype=np.float32)
        out[:, new_of_prov] = pts.astype(np.float32)
        self.points = out
        self._lat = lat

    # -------------------------------------------------------------- interface
    def n_nodes(self, l=None) -> int:
        return self._n_nodes[self.L if l is None else int(l)]

    def elements(self, l=None) -> np.ndarray:
        """sshex8 connectivity at level ``l``: int32 ``[(l+1)^3, E]`` (lidx order)."""
        l = self.L if l is None else int(l)
        if l not in self.levels:
            raise ValueError(f"level {l} not in hierarchy {self.levels}")
        if l not in self._elements:
            s = self.L // l
            n = l + 1
            zi, yi, xi = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
            v = sshex8_lidx(self.L, xi.reshape(-1) * s, yi.reshape(-1) * s, zi.reshape(-1) * s)
            el = np.ascontiguousarray(self._fine[v].astype(np.int32))
            assert el.max() < self.n_nodes(l)
            self._elements[l] = el
        return self._elements[l]

    def hex8_elements(self) -> np.ndarray:
        el1 = self.elements(1)
        return np.ascontiguousarray(el1[[sshex8_lidx(1, *HEX8_CORNERS[k]) for k in range(8)]])

    def macro_corner_lidx(self, l=None):
        l = self.L if l is None else l
        return [sshex8_lidx(l, *(HEX8_CORNERS[k] * l)) for k in range(8)]

    def boundary_names(self):
        return list(self._boundary)

    def boundary_nodes(self, name: str, l=None) -> np.ndarray:
        """Sorted node ids (< n_nodes(l)) on the boundary faces whose corners are all in
        the macro node set ``name``."""
        l = self.L if l is None else int(l)
        if name not in self._boundary:
            raise KeyError(f"no boundary node set {name!r} (have {sorted(self._boundary)})")
        inset = np.zeros(int(self._hex.max()) + 1, dtype=bool)
        ids = self._boundary[name]
        inset[ids[ids <= self._hex.max()]] = True
        L, s = self.L, self.L // l
        out = []
        for f, (d, side) in enumerate(_FACES):
            cs = [c for c in range(8) if HEX8_CORNERS[c, d] == side]
            on = inset[self._hex[cs]].all(axis=0)
            on &= self._face_multiplicity[f] == 1
            if not on.any():
                continue
            pts = np.flatnonzero((self._lat[d] == side * L) & ((self._lat % s) == 0).all(axis=0))
            out.append(self._fine[np.ix_(pts, np.flatnonzero(on))].reshape(-1))
        if not out:
            return np.zeros(0, dtype=np.int32)
        return np.unique(np.concatenate(out)).astype(np.int32)

    def all_boundary_nodes(self, l=None) -> np.ndarray:
        return np.unique(np.concatenate([self.boundary_nodes(k, l) for k in self._boundary])).astype(np.int32)


def ssmesh_from_folder(folder, L: int) -> HexSSMesh:
    """Read a reference HEX8 mesh folder and refine it to level ``L``."""
    m = read_sfem_mesh(folder)
    if m.element_type.upper() not in ("HEX8", "HEXAHEDRON", "HEX"):
        raise ValueError(f"{folder}: element type {m.element_type} (HEX8 meshes only)")
    return HexSSMesh(m.elements, m.points, L, boundary=m.boundary_nodes)


def sshex8_to_hex8(elements: np.ndarray, L: int) -> np.ndarray:
    """Micro hex8 connectivity ``[8, E * L^3]`` (standard corner order) of a level-``L``
    sshex8 connectivity ``[(L+1)^3, E]``: micro element ``m = xi + L (yi + L zi)`` of
    macro element ``e`` is column ``e * L^3 + m``.  With the fine points this is a plain
    HEX8 mesh (e.g. to write with :func:`write_sfem_mesh` for the reference)."""
    el = np.asarray(elements)
    if el.shape[0] != (L + 1) ** 3:
        raise ValueError(f"connectivity has {el.shape[0]} rows, level {L} needs {(L + 1) ** 3}")
    zi, yi, xi = np.meshgrid(np.arange(L), np.arange(L), np.arange(L), indexing="ij")
    xi, yi, zi = xi.reshape(-1), yi.reshape(-1), zi.reshape(-1)
    # keep the ids' own integer type (the mesh folders may carry int64 ids)
    out = np.empty((8, el.shape[1], L ** 3), dtype=el.dtype)
    for c in range(8):
        dx, dy, dz = HEX8_CORNERS[c]
        out[c] = el[sshex8_lidx(L, xi + dx, yi + dy, zi + dz)].T
    return np.ascontiguousarray(out.reshape(8, -1))
