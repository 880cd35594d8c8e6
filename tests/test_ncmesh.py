"""Host logic of nonconforming meshes: the classification of hanging faces by
``rkdg3d_gb300/csrc/rkdg_ncmesh.cpp`` (slave faces paired with the coarse
element whose face contains them, master faces checked for coverage, holes
refused), run on the CPU through the C++ driver ``tests/ncmesh_check.cpp``
and compared with a brute-force geometric pairing written here: every lone
face (a face no second element shares and no boundary element lists) whose
corners all lie on a larger lone face of another element is a slave of that
element."""
import json
import os
import shutil
import subprocess

import numpy as np
import pytest

from rkdg3d_gb300 import mesh as M

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "rkdg3d_gb300", "csrc")

# MFEM local face vertex lists per geometry
FACES = {M.GEOM_TRIANGLE: [(0, 1), (1, 2), (2, 0)],
         M.GEOM_SQUARE: [(0, 1), (1, 2), (2, 3), (3, 0)],
         M.GEOM_CUBE: [(3, 2, 1, 0), (0, 1, 5, 4), (1, 2, 6, 5), (2, 3, 7, 6), (3, 0, 4, 7), (4, 5, 6, 7)]}


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ not available")
    exe = str(tmp_path_factory.mktemp("ncmesh") / "check")
    subprocess.run([gxx, "-O2", "-std=c++17", "-I", CSRC, os.path.join(HERE, "ncmesh_check.cpp"),
                    os.path.join(CSRC, "rkdg_ncmesh.cpp"), os.path.join(CSRC, "rkdg_refelem.cpp"),
                    "-o", exe], check=True)
    return exe


def lone_faces(m):
    faces = FACES[m.geom]
    count = {}
    for e in range(m.num_elements):
        for lf, fv in enumerate(faces):
            key = tuple(sorted(m.elem_vertices[e, list(fv)]))
            count.setdefault(key, []).append((e, lf))
    bdr = {tuple(sorted(r)) for r in m.bdr_vertices.tolist()}
    return sorted(v[0] for k, v in count.items() if len(v) == 1 and k not in bdr)


def corners(m, e, lf):
    return m.elem_coords[e, list(FACES[m.geom][lf])]


def measure(c):
    if len(c) == 2:
        return float(np.linalg.norm(c[1] - c[0]))
    return float(np.linalg.norm(np.cross(c[1] - c[0], c[3] - c[0])))


def on_face(p, c, tol=1e-9):
    """Point p on the closed segment / parallelogram with corners c."""
    d = p - c[0]
    if len(c) == 2:
        u = c[1] - c[0]
        uu = float(u @ u)
        t = float(d @ u) / uu
        return abs(u[0] * d[1] - u[1] * d[0]) <= tol * uu and -tol <= t <= 1 + tol
    u, v = c[1] - c[0], c[3] - c[0]
    n = np.cross(u, v)
    if abs(float(d @ n)) > tol * float(n @ n):
        return False
    st = np.linalg.lstsq(np.stack([u, v], axis=1), d, rcond=None)[0]
    return bool(np.all(st >= -tol) and np.all(st <= 1 + tol))


def brute_force(m, lone):
    out = set()
    for e, lf in lone:
        ca = corners(m, e, lf)
        found = [(e2, lf2) for e2, lf2 in lone
                 if e2 != e and measure(corners(m, e2, lf2)) > measure(ca) * (1 + 1e-9)
                 and all(on_face(p, corners(m, e2, lf2)) for p in ca)]
        assert len(found) <= 1, (e, lf, found)
        if found:
            out.add((e, lf, *found[0]))
    return out


def classify(checker, tmp_path, m):
    lone = lone_faces(m)
    ne, nv, dim = m.elem_coords.shape
    vi = [1, 2 if m.geom == M.GEOM_TRIANGLE else 3, 4][:dim]
    J = np.zeros((ne, 9))
    X0 = m.elem_coords[:, 0]
    for i in range(dim):
        for r in range(dim):
            J[:, i * dim + r] = m.elem_coords[:, vi[r], i] - X0[:, i]
    nf = len(FACES[m.geom])
    fmeas = np.array([[measure(corners(m, e, lf)) for e in range(ne)] for lf in range(nf)])
    path = tmp_path / "mesh.bin"
    with open(path, "wb") as fh:
        np.array([dim, m.geom, nv, ne, len(lone)], np.int32).tofile(fh)
        np.ascontiguousarray(m.elem_coords, np.float64).tofile(fh)
        J.tofile(fh)
        np.ascontiguousarray(fmeas, np.float64).tofile(fh)
        np.array(lone, np.int32).reshape(-1, 2).tofile(fh)
    r = subprocess.run([checker, str(path)], capture_output=True, text=True, check=True)
    return json.loads(r.stdout), lone


def _two_level_quads():
    m, ch = M.refine_nc(M.quad_grid(6, 6), [14], return_children=True)
    return M.refine_nc(m, [ch[14][1]])  # a child next to the coarse element on its right


MESHES = {
    "quad periodic": lambda: M.refine_nc(M.quad_grid(8, 8, periodic=(True, True)), [9, 10, 18, 45]),
    "quad two levels": _two_level_quads,
    "tri": lambda: M.refine_nc(M.tri_grid(6, 6, 0, 1, 0, 1, jitter=0.2, seed=3), [14, 15, 30]),
    "hex periodic": lambda: M.refine_nc(M.hex_grid(4, 4, 4), [21, 22, 42]),
    "hex walled": lambda: M.refine_nc(M.hex_grid(4, 4, 4, periodic=(False,) * 3), [21, 5, 63]),
}


@pytest.mark.parametrize("name", sorted(MESHES))
def test_classification_matches_brute_force(checker, tmp_path, name):
    m = MESHES[name]()
    res, lone = classify(checker, tmp_path, m)
    assert res["ok"], res
    got = {tuple(s) for s in res["slaves"]}
    assert len(got) == len(res["slaves"])  # each slave once
    assert got == brute_force(m, lone)
    # every lone face is a slave or a master that some slave names
    masters = {(s[2], s[3]) for s in got}
    assert {(s[0], s[1]) for s in got} | masters == set(lone)
    if name == "quad two levels":  # quarter-length slaves on a coarse face
        ratios = {round(measure(corners(m, s[2], s[3])) / measure(corners(m, s[0], s[1]))) for s in got}
        assert ratios == {2, 4}


def test_conforming_mesh_has_no_lone_faces(checker, tmp_path):
    res, lone = classify(checker, tmp_path, M.hex_grid(3, 3, 3, periodic=(False,) * 3))
    assert lone == [] and res == {"ok": True, "slaves": []}


def test_hole_is_refused(checker, tmp_path):
    """Faces around a missing element have no neighbour, no boundary element
    and no hanging faces covering them."""
    m = M.refine_nc(M.quad_grid(6, 6, periodic=(True, True)), [8])
    keep = [e for e in range(m.num_elements) if e != 21]
    holed = M.Mesh(2, m.geom, m.elem_vertices[keep], m.elem_coords[keep], m.bdr_vertices, m.bdr_attr)
    res, _ = classify(checker, tmp_path, holed)
    assert not res["ok"] and res["error"]
