"""Case directories (settings.yml + Gmsh v2.2 mesh): the settings parser, the
case loader's restatement of CaseManager's set-up (initial fields, boundary
patches by physical name, limiter, time scheme), its refusals, and the VTU
writer.  The GPU run of a case against the oracle is in
tests/test_gpu_casefile.py."""
import os
import xml.etree.ElementTree as ET

import numpy as np
import pytest

from rkdg3d_gb300 import casefile as CF
from rkdg3d_gb300 import mesh as M
from rkdg3d_gb300.solver import (BC_OPEN, BC_SLIP, BC_SUPERSONIC_INLET, IND_BJ, LIM_MULTI,
                                 TABLEAU_REFERENCE_RK2)

# the reference's cases/ directory, where a checkout is at hand
REF_CASES = os.environ.get("RKDG_REFERENCE_CASES", "")


def write_msh22(path, nx, ny, x1=1.0, y1=0.1):
    """A structured nx x ny quadrilateral mesh of [0, x1] x [0, y1] as a Gmsh
    v2.2 ASCII file with physical lines bottom(1) right(2) top(3) left(4) and
    the physical surface Fluid(5)."""
    vid = lambda i, j: 1 + i + (nx + 1) * j
    nodes = [(vid(i, j), x1 * i / nx, y1 * j / ny) for j in range(ny + 1) for i in range(nx + 1)]
    el = []
    for i in range(nx):
        el.append((1, 1, [vid(i, 0), vid(i + 1, 0)]))
        el.append((1, 3, [vid(i + 1, ny), vid(i, ny)]))
    for j in range(ny):
        el.append((1, 2, [vid(nx, j), vid(nx, j + 1)]))
        el.append((1, 4, [vid(0, j + 1), vid(0, j)]))
    for j in range(ny):
        for i in range(nx):
            el.append((3, 5, [vid(i, j), vid(i + 1, j), vid(i + 1, j + 1), vid(i, j + 1)]))
    with open(path, "w") as fh:
        fh.write("$MeshFormat\n2.2 0 8\n$EndMeshFormat\n$PhysicalNames\n5\n")
        for dim, tag, name in [(1, 1, "bottom"), (1, 2, "right"), (1, 3, "top"), (1, 4, "left"),
                               (2, 5, "Fluid")]:
            fh.write(f'{dim} {tag} "{name}"\n')
        fh.write(f"$EndPhysicalNames\n$Nodes\n{len(nodes)}\n")
        for n, x, y in nodes:
            fh.write(f"{n} {x!r} {y!r} 0\n")
        fh.write(f"$EndNodes\n$Elements\n{len(el)}\n")
        for k, (t, tag, vs) in enumerate(el):
            fh.write(f"{k + 1} {t} 2 {tag} {tag} {' '.join(map(str, vs))}\n")
        fh.write("$EndElements\n")


SETTINGS = """### a Sod tube in the reference's settings format
mesh:
    file: tube.msh
    serialRefLevels: 0
    adaptive: 0

physics:
    type:   perfectGas
    gamma:  1.4
    R:      1.0

internalField:
    type:       planeBreakup
    origin:     [0.5,0,0]
    normal:     [1,0,0]
    left:
        rho:    1.0
        U:      [0,0,0]
        p:      1.0
    right:
        rho:    0.125
        U:      [0,0,0]
        p:      0.1

boundaryField:
    left:   # inlet
        type:   supersonicInlet
        rhoI:   1.0
        UI:     [0.5,0.1,0.3]
        pI:     1.0
    right:
        type:   outlet
    top:
        type:   slip
    bottom:
        type:   slip
    nowhere:
        type:   slip

spatial:
    polyOrder:      1
    riemannSolver:  HLLC
    limiter:
        type:       Multi
        indicator:  BJ

time:
    order:  2
    tEnd:   0.01
    dt:     0.001
    type:   dynamic
    CoMax:  0.2
"""


@pytest.fixture
def tube(tmp_path):
    write_msh22(tmp_path / "tube.msh", 40, 2)
    (tmp_path / "settings.yml").write_text(SETTINGS)
    return str(tmp_path)


def test_parse_settings():
    s = CF.parse_settings(SETTINGS)
    assert s["mesh"]["file"] == "tube.msh" and s["mesh"]["adaptive"] == 0
    assert s["internalField"]["origin"] == [0.5, 0, 0]
    assert s["internalField"]["right"]["rho"] == 0.125
    assert s["boundaryField"]["left"]["type"] == "supersonicInlet"  # comment stripped
    assert s["spatial"]["limiter"]["indicator"] == "BJ"
    assert s["time"]["CoMax"] == 0.2


def test_load_case(tube):
    case = CF.load_case(tube)
    assert case.mesh.num_elements == 80 and case.order == 1
    bcs = {a: (t, st) for a, t, st in case.bcs}
    # patches map through the physical names; an unknown name is skipped
    assert set(bcs) == {1, 2, 3, 4}
    assert bcs[3][0] == BC_SLIP and bcs[2][0] == BC_OPEN and bcs[4][0] == BC_SUPERSONIC_INLET
    rho, u, v, p = 1.0, 0.5, 0.1, 1.0
    # the reference's inlet energy: p/(gamma-1) + rho (u^2 + v^2)/2
    assert np.allclose(bcs[4][1], [rho, rho * u, rho * v, p / 0.4 + 0.5 * rho * (u * u + v * v)])
    assert case.limiter[:2] == (LIM_MULTI, IND_BJ)
    assert case.tableau == TABLEAU_REFERENCE_RK2 and case.dt_mode == 0 and case.cfl == 0.2
    X = np.array([[0.25, 0.75], [0.05, 0.05]])
    rho, u, v, p = case.ic(X)
    assert np.allclose(rho, [1.0, 0.125]) and np.allclose(p, [1.0, 0.1])


def test_initial_field_known_answers():
    sph = CF.initial_field({"type": "sphericalBreakup", "origin": [0, 0, 0], "radius": 1.0,
                            "left": {"rho": 2.0, "U": [0, 0, 0], "p": 3.0},
                            "right": {"rho": 1.0, "U": [0, 0, 0], "p": 1.0}}, 2, 1.4)
    r = np.array([0.5, 1.01, 1.05])  # inside, inside the band (r^2 < 1.04), outside it
    rho, u, v, p = sph(np.stack([r, 0 * r]))
    ramp = (1.01 - 1.0) * (1.0 - 2.0) / 0.2 + 2.0
    assert np.allclose(rho, [2.0, ramp, 1.0])
    pulse = CF.initial_field({"type": "densityPulse", "origin": [0, 0, 0], "epsilon": 5.0,
                              "U": [1, 0, 0], "p": 1.0}, 2, 1.4)
    rho = pulse(np.array([[0.3], [0.4]]))[0]
    want = (1 - 0.4 * 25 * np.exp(0.25 - 1) / (8 * 1.4 * 3.14169265 ** 2)) ** (1 / 0.4)
    assert np.allclose(rho, want, rtol=1e-14)


@pytest.mark.parametrize("edit,msg", [
    (("spatial", "limiter", "type", "BJ"), "limiter type"),
    (("boundaryField", "right", "type", "subsonicInlet"), "boundary condition type"),
    (("mesh", "adaptive", None, 1), "adaptive"),
    (("time", "order", None, 4), "time order"),
    (("spatial", "riemannSolver", None, "Roe"), "Riemann solver")])
def test_refusals(tube, edit, msg):
    """Settings the reference exits on (or that need MFEM) are refused."""
    s = CF.read_settings(os.path.join(tube, "settings.yml"))
    a, b, c, val = edit
    if c is None:
        s[a][b] = val
    else:
        s[a][b][c] = val
    with pytest.raises(CF.CaseError, match=msg):
        CF.load_case(tube, s)


def test_char_outlet_factory(tube):
    """charOutlet (case_manager.cpp:779-802): the outer state from rhoI, UI,
    pI; the energy omits the third velocity component, and in 2D it takes the
    slot the reference first fills with rho w."""
    from rkdg3d_gb300.solver import BC_CHAR_OUTLET
    s = CF.read_settings(os.path.join(tube, "settings.yml"))
    s["boundaryField"]["right"] = {"type": "charOutlet", "rhoI": 0.8, "UI": [0.3, 0.1, 0.2], "pI": 0.7}
    case = CF.load_case(tube, s)
    t, st = [(t, st) for a, t, st in case.bcs if t == BC_CHAR_OUTLET][0]
    rho, u, v = 0.8, 0.3, 0.1
    assert np.allclose(st, [rho, rho * u, rho * v, 0.7 / 0.4 + 0.5 * rho * (u * u + v * v)], rtol=1e-15)


def test_serial_refinement(tube):
    s = CF.read_settings(os.path.join(tube, "settings.yml"))
    s["mesh"]["serialRefLevels"] = 1
    case = CF.load_case(tube, s)
    assert case.mesh.num_elements == 320
    assert len(case.mesh.bdr_attr) == 2 * (2 * 40 + 2 * 2)  # every boundary face split in two


def test_write_vtu(tube, tmp_path):
    case = CF.load_case(tube)
    ne = case.mesh.num_elements
    means = np.stack([np.full(ne, 1.0), np.full(ne, 0.2), np.zeros(ne), np.full(ne, 2.5)])
    path = str(tmp_path / "out.vtu")
    CF.write_vtu(path, case.mesh, means)
    root = ET.parse(path).getroot()
    piece = root.find("UnstructuredGrid/Piece")
    assert int(piece.get("NumberOfCells")) == ne
    arrays = {a.get("Name"): np.array(a.text.split(), float) for a in piece.iter("DataArray")
              if a.get("Name")}
    assert np.allclose(arrays["p"], 0.4 * (2.5 - 0.5 * 0.2 * 0.2))
    assert np.allclose(arrays["U"].reshape(-1, 3)[:, 0], 0.2)


@pytest.mark.skipif(not REF_CASES or not os.path.isdir(REF_CASES),
                    reason="RKDG_REFERENCE_CASES not set")
def test_reference_settings_parse():
    """Every settings.yml the reference ships parses."""
    n = 0
    for d in sorted(os.listdir(REF_CASES)):
        p = os.path.join(REF_CASES, d, "settings.yml")
        if os.path.exists(p):
            s = CF.read_settings(p)
            assert {"mesh", "physics", "internalField", "spatial", "time"} <= set(s)
            n += 1
    assert n > 10


def test_restart_frame_round_trip(tube, tmp_path):
    """A restart frame keeps mesh, order, state, time, cycle and time step
    exactly; a missing frame is refused as the reference refuses it."""
    case = CF.load_case(tube)
    x = np.random.default_rng(3).normal(size=4 * 4 * case.mesh.num_elements)
    out = tmp_path / "frames"
    out.mkdir()
    name = CF.save_restart(str(out), 40, 0.0123, 4.5e-4, case.mesh, case.order, x)
    assert name == "restart_000040"
    assert (out / "restart_000040" / "mesh.npz").exists() and (out / "restart_000040.json").exists()
    fr = CF.load_restart(str(out), 40)
    assert fr["cycle"] == 40 and fr["time"] == 0.0123 and fr["time_step"] == 4.5e-4
    assert fr["order"] == case.order and np.array_equal(fr["x"], x)
    m = fr["mesh"]
    assert m.dim == case.mesh.dim and m.geom == case.mesh.geom
    for f in ("elem_vertices", "elem_coords", "bdr_vertices", "bdr_attr"):
        assert np.array_equal(getattr(m, f), getattr(case.mesh, f))
    with pytest.raises(CF.CaseError, match="Error loading data collection"):
        CF.load_restart(str(out), 41)


def test_restart_frame_queue(tube, tmp_path):
    """initializeRestartQueue / cleanPreviousRestartFrames: frames later than
    the restarted cycle are removed at start, then the n newest are kept;
    other files are left alone."""
    case = CF.load_case(tube)
    x = np.zeros(4 * 4 * case.mesh.num_elements)
    out = str(tmp_path)
    for c in (0, 10, 20, 30):
        CF.save_restart(out, c, 0.1 * c, 1e-3, case.mesh, case.order, x)
    fq = CF.RestartFrames(out, 2, restart_cycle=20)
    assert fq.queue == ["restart_000000", "restart_000010", "restart_000020"]
    assert not os.path.exists(os.path.join(out, "restart_000030"))
    assert not os.path.exists(os.path.join(out, "restart_000030.json"))
    CF.save_restart(out, 25, 2.5, 1e-3, case.mesh, case.order, x)
    fq.saved(25)
    # one removal per save, the oldest (the reference pops once when the
    # queue is longer than nSavedFrames)
    assert fq.queue == ["restart_000010", "restart_000020", "restart_000025"]
    assert not os.path.exists(os.path.join(out, "restart_000000"))
    assert os.path.exists(os.path.join(tube, "settings.yml")) and os.path.exists(
        os.path.join(tube, "tube.msh"))
    names = sorted(e for e in os.listdir(out) if e.startswith("restart_") and not e.endswith(".json"))
    assert names == fq.queue
