"""Host logic of the shared-face hexahedral kernel: the per-CTA schedules
(Morton grouping of the elements, face rounds) built by
``rkdg3d_gb300/csrc/rkdg_hexsched.cpp``, checked on the CPU by the C++ driver
``tests/hex_schedule_check.cpp`` for structured, bounded, shuffled and
rotated meshes and for an interior-face graph with an odd cycle."""
import json
import os
import shutil
import subprocess

import numpy as np
import pytest

from rkdg3d_gb300 import mesh as M

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "rkdg3d_gb300", "csrc")

# MFEM hexahedron local faces (vertex lists)
HEX_FACES = [(0, 1, 2, 3), (0, 1, 5, 4), (1, 2, 6, 5), (2, 3, 7, 6), (3, 0, 4, 7), (4, 5, 6, 7)]


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ not available")
    exe = str(tmp_path_factory.mktemp("hexsched") / "check")
    subprocess.run([gxx, "-O2", "-std=c++17", "-I", CSRC, os.path.join(HERE, "hex_schedule_check.cpp"),
                    os.path.join(CSRC, "rkdg_hexsched.cpp"), "-o", exe], check=True)
    return exe


def face_tables(ev):
    """fnbr / fcode [6][ne] as the library builds them: Elem1 = the first
    (element, local face) owning a face, code = other local face | side << 3."""
    ne = ev.shape[0]
    fnbr = np.full((6, ne), -1, np.int32)
    fcode = np.zeros((6, ne), np.int32)
    first = {}
    for e in range(ne):
        for lf, fv in enumerate(HEX_FACES):
            key = tuple(sorted(ev[e, list(fv)]))
            if key in first:
                e1, lf1 = first[key]
                fnbr[lf1, e1], fnbr[lf, e] = e, e1
                fcode[lf1, e1] = lf
                fcode[lf, e] = lf1 | 8
            else:
                first[key] = (e, lf)
    return fnbr, fcode


def run(checker, tmp_path, coords, fnbr, fcode):
    ne = fnbr.shape[1]
    path = tmp_path / "mesh.bin"
    with open(path, "wb") as fh:
        np.array([ne, 8], np.int32).tofile(fh)
        np.ascontiguousarray(coords, np.float64).tofile(fh)
        np.ascontiguousarray(fnbr, np.int32).tofile(fh)
        np.ascontiguousarray(fcode, np.int32).tofile(fh)
    out = subprocess.run([checker, str(path)], capture_output=True, text=True)
    res = json.loads(out.stdout.strip().splitlines()[-1])
    assert out.returncode == 0 and res["ok"], res
    return res


def cube_rotations():
    """The 24 proper rotations of the unit cube as permutations of MFEM's
    vertex order."""
    offs = np.array([(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0), (0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1)])
    c = offs - 0.5
    perms = []
    import itertools
    for p in itertools.permutations(range(3)):
        for s in itertools.product([1, -1], repeat=3):
            R = np.zeros((3, 3))
            for i in range(3):
                R[i, p[i]] = s[i]
            if np.linalg.det(R) < 0:
                continue
            rc = c @ R.T
            perms.append([int(np.argmin(np.abs(c - v).sum(1))) for v in rc])
    return np.array(perms)


@pytest.mark.parametrize("n,periodic", [(3, True), (4, True), (8, True), (5, False), (7, False)])
def test_structured(checker, tmp_path, n, periodic):
    m = M.hex_grid(n, n, n, periodic=(periodic,) * 3)
    fnbr, fcode = face_tables(m.elem_vertices)
    res = run(checker, tmp_path, m.elem_coords, fnbr, fcode)
    assert res["built"]
    if n == 3 and periodic:
        # a CTA holds whole periodic rings of three elements (odd cycles):
        # one extra round, and rounds that mix axes
        assert 6 < res["max_rounds"] <= 8
        return
    assert res["max_rounds"] == 6
    # consistently oriented: every round visits faces of one normal axis
    assert res["mixed_rounds"] == 0
    if n == 8:
        # 2^3 mesh: every run of 24 elements is three 2x2x2 octants
        assert res["inside_sides"] >= 0.55 * 6 * n ** 3


def test_shuffled_and_rotated(checker, tmp_path):
    """Element order shuffled and each element's local numbering rotated:
    the grouping and rounds depend only on the face tables and centres."""
    rng = np.random.default_rng(5)
    m = M.hex_grid(6, 5, 7, periodic=(True, False, True))
    order = rng.permutation(m.num_elements)
    rots = cube_rotations()
    assert len(rots) == 24
    pick = rots[rng.integers(0, 24, m.num_elements)]
    ev = np.take_along_axis(m.elem_vertices[order], pick, 1)
    ec = np.take_along_axis(m.elem_coords[order], pick[:, :, None], 1)
    fnbr, fcode = face_tables(ev)
    res = run(checker, tmp_path, ec, fnbr, fcode)
    assert res["built"] and res["max_rounds"] == 6


def test_odd_cycle(checker, tmp_path):
    """Three elements pairwise adjacent (an odd cycle of interior faces, as
    around an edge of valence three): the colouring falls back to a third
    colour for the cycle and still visits every face once."""
    ne = 3
    fnbr = np.full((6, ne), -1, np.int32)
    fcode = np.zeros((6, ne), np.int32)

    def link(e1, lf1, e2, lf2):
        fnbr[lf1, e1], fnbr[lf2, e2] = e2, e1
        fcode[lf1, e1] = lf2
        fcode[lf2, e2] = lf1 | 8

    link(0, 2, 1, 4)
    link(1, 3, 2, 1)
    link(0, 3, 2, 4)
    rng = np.random.default_rng(1)
    coords = rng.uniform(0, 1, (ne, 8, 3))
    res = run(checker, tmp_path, coords, fnbr, fcode)
    assert res["built"] and res["inside_sides"] == 6
