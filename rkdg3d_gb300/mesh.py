"""Host-side mesh descriptions for the RKDG C ABI.

The reference keeps mesh I/O, boundary set-up and refinement on the host in
MFEM (``case_manager.cpp:217-297``); the GPU path only needs, after every
adapt, the element-to-vertex topology (periodic seams share vertex ids), each
element's own corner coordinates and the boundary faces with their 1-based
attributes.  This module builds that description for the structured meshes of
the benchmark cases and reads Gmsh v2.2 ASCII files like the reference's
shipped fixtures.  Vertex orders follow MFEM: quads counter-clockwise,
hexahedra bottom face counter-clockwise then top face, triangles
counter-clockwise.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

GEOM_TRIANGLE = 2
GEOM_SQUARE = 3
GEOM_CUBE = 5

_NV = {GEOM_TRIANGLE: 3, GEOM_SQUARE: 4, GEOM_CUBE: 8}
_NVF = {GEOM_TRIANGLE: 2, GEOM_SQUARE: 2, GEOM_CUBE: 4}


@dataclass
class Mesh:
    dim: int
    geom: int
    elem_vertices: np.ndarray  # (ne, nv) int32 topological vertex ids
    elem_coords: np.ndarray    # (ne, nv, dim) float64 element corner coordinates
    bdr_vertices: np.ndarray   # (nb, nvf) int32
    bdr_attr: np.ndarray       # (nb,) int32, 1-based

    @property
    def num_elements(self) -> int:
        return int(self.elem_vertices.shape[0])

    def validate(self) -> None:
        nv = _NV[self.geom]
        assert self.elem_vertices.shape == (self.num_elements, nv)
        assert self.elem_coords.shape == (self.num_elements, nv, self.dim)
        assert self.bdr_vertices.shape[1:] == (_NVF[self.geom],)
        assert self.bdr_attr.shape == (self.bdr_vertices.shape[0],)

    def contiguous(self) -> "Mesh":
        return Mesh(self.dim, self.geom,
                    np.ascontiguousarray(self.elem_vertices, dtype=np.int32),
                    np.ascontiguousarray(self.elem_coords, dtype=np.float64),
                    np.ascontiguousarray(self.bdr_vertices.reshape(-1, _NVF[self.geom]), dtype=np.int32),
                    np.ascontiguousarray(self.bdr_attr, dtype=np.int32))


def quad_grid(nx: int, ny: int, x0=0.0, x1=1.0, y0=0.0, y1=1.0,
              periodic=(False, False)) -> Mesh:
    """Structured nx x ny quadrilateral mesh; element e = i + nx*j.
    Boundary attributes as MFEM's Cartesian meshes: 1 bottom, 2 right,
    3 top, 4 left (periodic directions have none)."""
    px, py = periodic
    nvx = nx if px else nx + 1
    nvy = ny if py else ny + 1
    xs = x0 + (x1 - x0) * np.arange(nx + 1) / nx
    ys = y0 + (y1 - y0) * np.arange(ny + 1) / ny

    def vid(i, j):
        return (i % nvx) + nvx * (j % nvy)

    I, J = np.meshgrid(np.arange(nx), np.arange(ny), indexing="xy")
    I = I.ravel()
    J = J.ravel()
    ev = np.stack([vid(I, J), vid(I + 1, J), vid(I + 1, J + 1), vid(I, J + 1)], axis=1)
    ec = np.stack([np.stack([xs[I], ys[J]], 1), np.stack([xs[I + 1], ys[J]], 1),
                   np.stack([xs[I + 1], ys[J + 1]], 1), np.stack([xs[I], ys[J + 1]], 1)], axis=1)
    bv, ba = [], []
    i = np.arange(nx)
    j = np.arange(ny)
    if not py:
        bv.append(np.stack([vid(i, 0), vid(i + 1, 0)], 1)); ba.append(np.full(nx, 1))
        bv.append(np.stack([vid(i + 1, ny), vid(i, ny)], 1)); ba.append(np.full(nx, 3))
    if not px:
        bv.append(np.stack([vid(nx, j), vid(nx, j + 1)], 1)); ba.append(np.full(ny, 2))
        bv.append(np.stack([vid(0, j + 1), vid(0, j)], 1)); ba.append(np.full(ny, 4))
    bv = np.concatenate(bv) if bv else np.zeros((0, 2), np.int32)
    ba = np.concatenate(ba) if ba else np.zeros((0,), np.int32)
    m = Mesh(2, GEOM_SQUARE, ev.astype(np.int32), ec.astype(np.float64), bv.astype(np.int32),
             ba.astype(np.int32))
    m.validate()
    return m


def hex_grid(nx: int, ny: int, nz: int, box=((0.0, 1.0), (0.0, 1.0), (0.0, 1.0)),
             periodic=(True, True, True)) -> Mesh:
    """Structured hexahedral mesh, element e = i + nx*(j + ny*k).  Boundary
    attributes as MFEM's Cartesian meshes: 1 z=min, 2 y=min, 3 x=max,
    4 y=max, 5 x=min, 6 z=max."""
    n = (nx, ny, nz)
    nv = [n[d] if periodic[d] else n[d] + 1 for d in range(3)]
    cs = [box[d][0] + (box[d][1] - box[d][0]) * np.arange(n[d] + 1) / n[d] for d in range(3)]

    def vid(i, j, k):
        return (i % nv[0]) + nv[0] * ((j % nv[1]) + nv[1] * (k % nv[2]))

    K, J, I = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    I, J, K = I.ravel(), J.ravel(), K.ravel()
    offs = [(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0), (0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1)]
    ev = np.stack([vid(I + a, J + b, K + c) for a, b, c in offs], 1)
    ec = np.stack([np.stack([cs[0][I + a], cs[1][J + b], cs[2][K + c]], 1) for a, b, c in offs], 1)
    bv, ba = [], []

    def add(quads, attr):
        bv.append(quads)
        ba.append(np.full(quads.shape[0], attr))

    a2, b2 = np.meshgrid(np.arange(nx), np.arange(ny), indexing="ij")
    a2, b2 = a2.ravel(), b2.ravel()
    if not periodic[2]:
        add(np.stack([vid(a2, b2 + 1, 0), vid(a2 + 1, b2 + 1, 0), vid(a2 + 1, b2, 0), vid(a2, b2, 0)], 1), 1)
        add(np.stack([vid(a2, b2, nz), vid(a2 + 1, b2, nz), vid(a2 + 1, b2 + 1, nz), vid(a2, b2 + 1, nz)], 1), 6)
    a2, c2 = np.meshgrid(np.arange(nx), np.arange(nz), indexing="ij")
    a2, c2 = a2.ravel(), c2.ravel()
    if not periodic[1]:
        add(np.stack([vid(a2, 0, c2), vid(a2 + 1, 0, c2), vid(a2 + 1, 0, c2 + 1), vid(a2, 0, c2 + 1)], 1), 2)
        add(np.stack([vid(a2 + 1, ny, c2), vid(a2, ny, c2), vid(a2, ny, c2 + 1), vid(a2 + 1, ny, c2 + 1)], 1), 4)
    b2, c2 = np.meshgrid(np.arange(ny), np.arange(nz), indexing="ij")
    b2, c2 = b2.ravel(), c2.ravel()
    if not periodic[0]:
        add(np.stack([vid(nx, b2, c2), vid(nx, b2 + 1, c2), vid(nx, b2 + 1, c2 + 1), vid(nx, b2, c2 + 1)], 1), 3)
        add(np.stack([vid(0, b2 + 1, c2), vid(0, b2, c2), vid(0, b2, c2 + 1), vid(0, b2 + 1, c2 + 1)], 1), 5)
    bv = np.concatenate(bv) if bv else np.zeros((0, 4), np.int32)
    ba = np.concatenate(ba) if ba else np.zeros((0,), np.int32)
    m = Mesh(3, GEOM_CUBE, ev.astype(np.int32), ec.astype(np.float64), bv.astype(np.int32),
             ba.astype(np.int32))
    m.validate()
    return m


def perturb(mesh: Mesh, amount: float, seed: int = 0) -> Mesh:
    """The mesh with every vertex that lies on no boundary face moved by
    U(-amount, amount) per coordinate (the same move for every element
    sharing the vertex): on a quad grid this gives general, non-parallelogram
    quadrilaterals.  Periodic seams keep their coordinates."""
    rng = np.random.default_rng(seed)
    nv = int(mesh.elem_vertices.max()) + 1
    shift = rng.uniform(-amount, amount, (nv, mesh.dim))
    fixed = np.zeros(nv, bool)
    fixed[mesh.bdr_vertices.ravel()] = True
    # vertices whose elements disagree on their position lie on a periodic seam
    first = {}
    for e in range(mesh.num_elements):
        for k, v in enumerate(mesh.elem_vertices[e]):
            x = mesh.elem_coords[e, k]
            if v in first and np.abs(first[v] - x).max() > 1e-12:
                fixed[v] = True
            first.setdefault(v, x)
    shift[fixed] = 0.0
    ec = mesh.elem_coords + shift[mesh.elem_vertices]
    m = Mesh(mesh.dim, mesh.geom, mesh.elem_vertices.copy(), ec, mesh.bdr_vertices.copy(),
             mesh.bdr_attr.copy())
    m.validate()
    return m


def tri_grid(nx: int, ny: int, x0=0.0, x1=1.0, y0=0.0, y1=1.0, jitter=0.0, seed=0) -> Mesh:
    """Structured grid with every quad split along its (i,j)-(i+1,j+1) diagonal
    into two counter-clockwise triangles (elements 2q, 2q+1 for quad q =
    i + nx*j).  Interior vertices are moved by U(-jitter*h, +jitter*h) per
    coordinate, drawn as ``numpy.random.default_rng(seed).uniform(-1, 1,
    (num_vertices, 2))`` in vertex order (only interior rows are applied).
    Boundary attributes: 1 bottom, 2 right, 3 top, 4 left."""
    nvx = nx + 1
    hx = (x1 - x0) / nx
    hy = (y1 - y0) / ny
    X, Y = np.meshgrid(x0 + hx * np.arange(nx + 1), y0 + hy * np.arange(ny + 1), indexing="xy")
    V = np.stack([X.ravel(), Y.ravel()], 1)
    if jitter:
        rng = np.random.default_rng(seed)
        d = rng.uniform(-1.0, 1.0, size=V.shape) * jitter * np.array([hx, hy])
        ii = np.arange(V.shape[0]) % nvx
        jj = np.arange(V.shape[0]) // nvx
        interior = (ii > 0) & (ii < nx) & (jj > 0) & (jj < ny)
        V[interior] += d[interior]

    def vid(i, j):
        return i + nvx * j

    I, J = np.meshgrid(np.arange(nx), np.arange(ny), indexing="xy")
    I, J = I.ravel(), J.ravel()
    v00, v10, v11, v01 = vid(I, J), vid(I + 1, J), vid(I + 1, J + 1), vid(I, J + 1)
    ev = np.empty((2 * I.size, 3), np.int64)
    ev[0::2] = np.stack([v00, v10, v11], 1)
    ev[1::2] = np.stack([v00, v11, v01], 1)
    ec = V[ev]
    i = np.arange(nx)
    j = np.arange(ny)
    bv = np.concatenate([np.stack([vid(i, 0), vid(i + 1, 0)], 1),
                         np.stack([vid(nx, j), vid(nx, j + 1)], 1),
                         np.stack([vid(i + 1, ny), vid(i, ny)], 1),
                         np.stack([vid(0, j + 1), vid(0, j)], 1)])
    ba = np.concatenate([np.full(nx, 1), np.full(ny, 2), np.full(nx, 3), np.full(ny, 4)])
    m = Mesh(2, GEOM_TRIANGLE, ev.astype(np.int32), ec.astype(np.float64), bv.astype(np.int32),
             ba.astype(np.int32))
    m.validate()
    return m


def read_gmsh22(path: str) -> Mesh:
    """Gmsh v2.2 ASCII reader for 2D triangle / quad and 3D hex meshes.  The
    boundary attribute is the element's physical tag.  Clockwise 2D elements
    are reordered counter-clockwise (MFEM fixes orientation on load)."""
    with open(path) as fh:
        lines = [ln.strip() for ln in fh]
    it = iter(range(len(lines)))
    nodes = {}
    elems = []
    k = 0
    while k < len(lines):
        if lines[k] == "$Nodes":
            n = int(lines[k + 1])
            for r in range(n):
                parts = lines[k + 2 + r].split()
                nodes[int(parts[0])] = [float(v) for v in parts[1:4]]
            k += n + 2
        elif lines[k] == "$Elements":
            n = int(lines[k + 1])
            for r in range(n):
                parts = [int(v) for v in lines[k + 2 + r].split()]
                etype, ntags = parts[1], parts[2]
                tags = parts[3:3 + ntags]
                verts = parts[3 + ntags:]
                elems.append((etype, tags[0] if tags else 0, verts))
            k += n + 2
        else:
            k += 1
    del it
    vol = {2: GEOM_TRIANGLE, 3: GEOM_SQUARE, 5: GEOM_CUBE}
    types = {e[0] for e in elems}
    geom = next(vol[t] for t in (5, 3, 2) if t in types)
    dim = 3 if geom == GEOM_CUBE else 2
    bdr_type = 3 if geom == GEOM_CUBE else 1
    ids = sorted(nodes)
    remap = {g: i for i, g in enumerate(ids)}
    coords = np.array([nodes[g][:dim] for g in ids], np.float64)
    vol_t = {GEOM_TRIANGLE: 2, GEOM_SQUARE: 3, GEOM_CUBE: 5}[geom]
    ev = np.array([[remap[v] for v in e[2]] for e in elems if e[0] == vol_t], np.int64)
    if dim == 2:
        p = coords[ev]
        a = p[:, 1] - p[:, 0]
        b = p[:, -1] - p[:, 0]
        cw = a[:, 0] * b[:, 1] - a[:, 1] * b[:, 0] < 0
        ev[cw] = ev[cw][:, ::-1]
    bv = np.array([[remap[v] for v in e[2]] for e in elems if e[0] == bdr_type], np.int64)
    ba = np.array([e[1] for e in elems if e[0] == bdr_type], np.int64)
    nvf = 4 if dim == 3 else 2
    m = Mesh(dim, geom, ev.astype(np.int32), coords[ev].astype(np.float64),
             bv.reshape(-1, nvf).astype(np.int32), ba.astype(np.int32))
    m.validate()
    return m


def read_gmsh22_physical_names(path: str) -> dict:
    """$PhysicalNames of a Gmsh v2.2 ASCII file: {name: (dimension, tag)}.  The
    reference maps each boundaryField patch name to its tag through this
    section (case_manager.cpp:299-448, 614-660)."""
    out = {}
    with open(path) as fh:
        lines = [ln.strip() for ln in fh]
    for k, ln in enumerate(lines):
        if ln == "$PhysicalNames":
            n = int(lines[k + 1])
            for r in range(n):
                parts = lines[k + 2 + r].split(maxsplit=2)
                out[parts[2].strip().strip('"')] = (int(parts[0]), int(parts[1]))
            break
    return out


# MFEM reference vertices and local faces of the tensor elements
_REF_VERT = {
    GEOM_SQUARE: np.array([(0, 0), (1, 0), (1, 1), (0, 1)], float),
    GEOM_CUBE: np.array([(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0),
                         (0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1)], float),
}
_LOCAL_FACES = {
    GEOM_SQUARE: [(0, 1), (1, 2), (2, 3), (3, 0)],
    GEOM_CUBE: [(3, 2, 1, 0), (0, 1, 5, 4), (1, 2, 6, 5), (2, 3, 7, 6), (3, 0, 4, 7), (4, 5, 6, 7)],
}


def refine_nc(mesh: Mesh, elements, return_children: bool = False):
    """Isotropic refinement of the listed quadrilaterals / hexahedra into
    2^dim children each, leaving their neighbours as they are: the result is
    a nonconforming mesh with hanging vertices, as MFEM's NC refinement
    (``Mesh::GeneralRefinement`` on a mesh made nonconforming by
    ``EnsureNCMesh``, ``case_manager.cpp:269``) produces.  New vertices are
    identified by the parent vertices they split (edge midpoints by the
    edge's two ids, face centres by the face's ids), so two refined
    neighbours share them and periodic identifications carry over.  A
    refined element is replaced by its first child; the others are
    appended.  Boundary faces of refined elements are split likewise.  With
    return_children, also {parent: [element of child c]} where child c sits
    at offset ((c >> d) & 1) / 2 along reference axis d of its parent."""
    geom = mesh.geom
    if geom == GEOM_TRIANGLE:
        return _refine_tri(mesh, elements, return_children)
    if geom not in _REF_VERT:
        raise ValueError("refine_nc supports triangles, quadrilaterals and hexahedra")
    dim = mesh.dim
    rv = _REF_VERT[geom]
    nv = rv.shape[0]
    ev = [list(r) for r in mesh.elem_vertices]
    ec = [np.array(r) for r in mesh.elem_coords]
    next_id = int(mesh.elem_vertices.max()) + 1
    keys = {}
    bdr = {tuple(sorted(r)): int(a) for r, a in zip(mesh.bdr_vertices.tolist(), mesh.bdr_attr.tolist())}
    new_bdr = {}

    def shape(r):  # multilinear shape functions at reference point r
        return np.prod([np.where(rv[:, d] > 0.5, r[d], 1.0 - r[d]) for d in range(dim)], axis=0)

    def vertex_id(pv, r):
        nonlocal next_id
        halves = [d for d in range(dim) if abs(r[d] - 0.5) < 1e-12]
        if not halves:  # parent corner
            k = int(np.argmin(np.abs(rv - r).sum(1)))
            return pv[k]
        # the parent vertices of the smallest entity (edge / face / cell) containing r
        fixed = [d for d in range(dim) if d not in halves]
        ids = [pv[k] for k in range(nv) if all(abs(rv[k, d] - r[d]) < 1e-12 for d in fixed)]
        key = (len(halves), tuple(sorted(ids)))  # the cell centre: all of the parent's ids
        if key not in keys:
            keys[key] = next_id
            next_id += 1
        return keys[key]

    children_of = {}
    for e in sorted(set(int(i) for i in elements)):
        pv, px = ev[e], ec[e]
        kids = []
        for c in range(2 ** dim):
            off = np.array([(c >> d) & 1 for d in range(dim)], float)
            rc = (rv + off) / 2.0  # child corners in the parent's reference space
            ids = [vertex_id(pv, r) for r in rc]
            xs = np.array([shape(r) @ px for r in rc])
            kids.append((ids, xs))
        children_of[e] = kids
        # split the parent's boundary faces
        for lf in _LOCAL_FACES[geom]:
            fk = tuple(sorted(pv[k] for k in lf))
            if fk not in bdr:
                continue
            attr = bdr.pop(fk)
            corner = rv[list(lf)]
            for c in range(2 ** (dim - 1)):
                # sub-face of the face: corners in the parent's reference space
                s_off = [(c >> d) & 1 for d in range(dim - 1)]
                e0 = corner[1] - corner[0]
                e1 = corner[-1] - corner[0] if dim == 3 else np.zeros(dim)
                pts = []
                for a, b in ([(0, 0), (1, 0), (1, 1), (0, 1)] if dim == 3 else [(0, 0), (1, 0)]):
                    pts.append(corner[0] + e0 * (s_off[0] + a) / 2 + (e1 * (s_off[1] + b) / 2 if dim == 3 else 0))
                new_bdr[tuple(sorted(vertex_id(pv, p) for p in pts))] = attr
    child_elems = {}
    for e, kids in children_of.items():
        ev[e], ec[e] = kids[0]
        child_elems[e] = [e]
        for ids, xs in kids[1:]:
            child_elems[e].append(len(ev))
            ev.append(ids)
            ec.append(xs)
    bdr.update(new_bdr)
    bv = np.array(list(bdr.keys()), np.int32).reshape(-1, _NVF[geom])
    ba = np.array(list(bdr.values()), np.int32)
    m = Mesh(dim, geom, np.array(ev, np.int32), np.array(ec, np.float64), bv, ba)
    m.validate()
    return (m, child_elems) if return_children else m


def _refine_tri(mesh: Mesh, elements, return_children: bool):
    """refine_nc for triangles: each listed triangle (v0, v1, v2) splits at
    its edge midpoints m01, m12, m20 into (v0, m01, m20), (m01, v1, m12),
    (m20, m12, v2) and the centre (m12, m20, m01), all counter-clockwise."""
    ev = [list(r) for r in mesh.elem_vertices]
    ec = [np.array(r) for r in mesh.elem_coords]
    next_id = int(mesh.elem_vertices.max()) + 1
    mids = {}
    bdr = {tuple(sorted(r)): int(a) for r, a in zip(mesh.bdr_vertices.tolist(), mesh.bdr_attr.tolist())}

    def mid(a, b):
        nonlocal next_id
        k = (min(a, b), max(a, b))
        if k not in mids:
            mids[k] = next_id
            next_id += 1
        return mids[k]

    child_elems = {}
    for e in sorted(set(int(i) for i in elements)):
        (a, b, c), (xa, xb, xc) = ev[e], ec[e]
        mab, mbc, mca = mid(a, b), mid(b, c), mid(c, a)
        pab, pbc, pca = (xa + xb) / 2, (xb + xc) / 2, (xc + xa) / 2
        kids = [([a, mab, mca], [xa, pab, pca]), ([mab, b, mbc], [pab, xb, pbc]),
                ([mca, mbc, c], [pca, pbc, xc]), ([mbc, mca, mab], [pbc, pca, pab])]
        for u, v, m in ((a, b, mab), (b, c, mbc), (c, a, mca)):
            attr = bdr.pop(tuple(sorted((u, v))), None)
            if attr is not None:
                bdr[tuple(sorted((u, m)))] = attr
                bdr[tuple(sorted((m, v)))] = attr
        ev[e], ec[e] = kids[0][0], np.array(kids[0][1])
        child_elems[e] = [e]
        for ids, xs in kids[1:]:
            child_elems[e].append(len(ev))
            ev.append(ids)
            ec.append(np.array(xs))
    bv = np.array(list(bdr.keys()), np.int32).reshape(-1, 2)
    ba = np.array(list(bdr.values()), np.int32)
    m = Mesh(2, GEOM_TRIANGLE, np.array(ev, np.int32), np.array(ec, np.float64), bv, ba)
    m.validate()
    return (m, child_elems) if return_children else m


def prolong_refined(x: np.ndarray, dim: int, order: int, ne_old: int, ne_new: int,
                    children: dict) -> np.ndarray:
    """Nodal DG state (byNODES, neq = dim + 2 variables) on the mesh before
    refine_nc -> the refined mesh: each child's nodal values are its
    parent's polynomial at the child's Gauss-Legendre nodes, the
    interpolation MFEM's GridFunction::Update applies to an L2 space after
    refinement (amr.cpp:45-46); exact, so cell integrals are conserved."""
    n1 = order + 1
    nd, neq = n1 ** dim, dim + 2
    t, _ = np.polynomial.legendre.leggauss(n1)
    x1 = (t + 1.0) / 2.0  # 1D GL nodes on [0, 1]

    def lagrange(s):  # l_i(s) for all i, s an array of points
        L = np.ones((len(s), n1))
        for i in range(n1):
            for m in range(n1):
                if m != i:
                    L[:, i] *= (s - x1[m]) / (x1[i] - x1[m])
        return L

    idx = np.stack(np.unravel_index(np.arange(nd), (n1,) * dim)[::-1], 1)  # node j -> (jx, jy, jz)
    xo = x.reshape(neq, ne_old, nd)
    xn = np.zeros((neq, ne_new, nd))
    xn[:, :ne_old] = xo
    for e, kids in children.items():
        for c, ce in enumerate(kids):
            off = np.array([(c >> d) & 1 for d in range(dim)], float)
            P = np.ones((nd, nd))
            for d in range(dim):
                Ld = lagrange((off[d] + x1[idx[:, d]]) / 2.0)  # child node -> parent basis along d
                P *= Ld[:, idx[:, d]]
            xn[:, ce] = xo[:, e] @ P.T
    return xn.reshape(-1)
