"""Host logic of the face-once tiled hexahedral kernel: the tiles (Morton
runs of 32 elements, per-axis face evaluations and halo lists) built by
``rkdg3d_gb300/csrc/rkdg_hexsched.cpp``, checked on the CPU by the C++
driver ``tests/hex_tile_check.cpp`` for structured, bounded, shuffled and
rotated meshes."""
import json
import os
import shutil
import subprocess

import numpy as np
import pytest

from rkdg3d_gb300 import mesh as M
from tests.test_hex_schedule import cube_rotations, face_tables

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "rkdg3d_gb300", "csrc")


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ not available")
    exe = str(tmp_path_factory.mktemp("hextile") / "check")
    subprocess.run([gxx, "-O2", "-std=c++17", "-I", CSRC, os.path.join(HERE, "hex_tile_check.cpp"),
                    os.path.join(CSRC, "rkdg_hexsched.cpp"), "-o", exe], check=True)
    return exe


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


@pytest.mark.parametrize("n,periodic", [(3, True), (4, True), (8, True), (16, True), (5, False),
                                        (12, True), (7, False)])
def test_structured(checker, tmp_path, n, periodic):
    m = M.hex_grid(n, n, n, periodic=(periodic,) * 3)
    fnbr, fcode = face_tables(m.elem_vertices)
    res = run(checker, tmp_path, m.elem_coords, fnbr, fcode)
    assert res["built"]
    if n in (8, 16):
        # 2^k mesh: every tile is a 4 x 4 x 2 block, 64 of its 192 face
        # sides face out: 3 + 1 = 4 evaluations per element
        assert res["evals_per_element"] == pytest.approx(4.0)
        assert res["max_halo"] == 32


def test_shuffled_and_rotated(checker, tmp_path):
    """Element order shuffled and each element's local numbering rotated:
    faces whose two local faces lie on different axes are evaluated from
    both sides through halos, every face side still once."""
    rng = np.random.default_rng(5)
    m = M.hex_grid(6, 5, 7, periodic=(True, False, True))
    order = rng.permutation(m.num_elements)
    pick = cube_rotations()[rng.integers(0, 24, m.num_elements)]
    ev = np.take_along_axis(m.elem_vertices[order], pick, 1)
    ec = np.take_along_axis(m.elem_coords[order], pick[:, :, None], 1)
    fnbr, fcode = face_tables(ev)
    res = run(checker, tmp_path, ec, fnbr, fcode)
    assert res["built"]
