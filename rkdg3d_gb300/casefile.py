"""Run the reference's case directories: ``settings.yml`` + a Gmsh v2.2 mesh.

The reference reads its cases through rapidyaml in ``CaseManager``
(``src/case_manager/case_manager.cpp``): mesh and refinement levels
(``loadMesh``, 217-297), physics (84-101), initial field (121-210, the
classes of ``src/initial_conditions/ic.hpp``), Riemann solver (523-543),
limiter (545-612), boundary patches matched to Gmsh physical names
(614-820), time scheme and stepping (822-895, 943-958).  This module
restates that set-up on top of the GPU context: ``load_case`` builds a
:class:`rkdg3d_gb300.cases.Case` from a case directory, ``run_case`` runs it
with ``rkdg_run`` (the time loop of ``main.cpp:509-553``), ``write_vtu``
writes cell means for ParaView.

Restart frames follow the reference's cycle (``main.cpp:453-495, 735-775``,
``CaseManager::loadMesh / loadInitialSolution / initializeRestartQueue /
cleanPreviousRestartFrames``): a frame before the loop and every
``postProcess.visSteps`` steps and at the end, named ``restart_<cycle>``, the
``time.nSavedFrames`` newest kept; ``time.restart`` continues from frame
``time.restartCycle`` with its mesh, state, time, cycle and time step.  The
frame contents are this module's own files (a NumPy mesh and state, a JSON
root) in place of MFEM's VisIt data collection, which needs MFEM.

Not restated: VisIt output for viewing, the adaptive refiner (``adaptive: 1``
is refused: its error estimator is MFEM's), parallel partitioning.  The
settings parser reads the subset of YAML the reference's files use: block
mappings by indentation, ``key: value`` scalars, ``[a, b, c]`` lists and
``#`` comments.
"""
from __future__ import annotations

import json
import os
import re
import shutil
from typing import Any

import numpy as np

from . import cases as C
from . import mesh as M
from .solver import (AVG_TRRS, BC_CHAR_OUTLET, BC_FIXED_PRESSURE_OUTLET, BC_OPEN, BC_SLIP,
                     BC_SUBSONIC_INLET_FIXED_PRESSURE, BC_SUBSONIC_INLET_TOTAL_PRESSURE,
                     BC_SUPERSONIC_INLET, BC_TOTAL_PRESSURE_OUTLET, FUN_MICHALAK, IND_BJ,
                     IND_EVERYWHERE, IND_NOWHERE, IND_SHU, LIM_FINDIFF, LIM_MULTI,
                     LIMITER_LINEARIZE, RS_HLL, RS_HLLC, RS_LLF, RS_RUSANOV,
                     TABLEAU_REFERENCE_RK2, TABLEAU_REFERENCE_RK3)


class CaseError(ValueError):
    """A setting the reference would reject (it prints and exits)."""


# ---- settings ---------------------------------------------------------------

def _scalar(text: str) -> Any:
    t = text.strip()
    if t.startswith("[") and t.endswith("]"):
        inner = t[1:-1].strip()
        return [_scalar(v) for v in inner.split(",")] if inner else []
    if len(t) >= 2 and t[0] == t[-1] and t[0] in "\"'":
        return t[1:-1]
    for conv in (int, float):
        try:
            return conv(t)
        except ValueError:
            pass
    if t in ("true", "True"):
        return True
    if t in ("false", "False"):
        return False
    return t


def _strip_comment(line: str) -> str:
    quote = None
    for i, ch in enumerate(line):
        if ch in "\"'":
            quote = None if quote == ch else (ch if quote is None else quote)
        elif ch == "#" and quote is None:
            return line[:i]
    return line


def parse_settings(text: str) -> dict:
    """The YAML subset of the reference's settings files -> nested dicts."""
    root: dict = {}
    stack = [(-1, root)]  # (indent, mapping)
    for raw in text.splitlines():
        line = _strip_comment(raw).rstrip()
        if not line.strip():
            continue
        indent = len(line) - len(line.lstrip(" "))
        key, sep, rest = line.strip().partition(":")
        if not sep:
            raise CaseError(f"cannot read settings line: {raw!r}")
        while stack and indent <= stack[-1][0]:
            stack.pop()
        parent = stack[-1][1]
        if rest.strip():
            parent[key.strip()] = _scalar(rest)
        else:
            child: dict = {}
            parent[key.strip()] = child
            stack.append((indent, child))
    return root


def read_settings(path: str) -> dict:
    with open(path) as fh:
        return parse_settings(fh.read())


# ---- initial fields (src/initial_conditions/ic.hpp) -------------------------

def _prim_state(d: dict, dim: int):
    """rho, velocity (dim components of U), p of a settings block.  In 2D the
    reference reads U[2] into the slot that p then overwrites, so only U[0],
    U[1] matter there."""
    u = [float(v) for v in d["U"]] + [0.0, 0.0, 0.0]
    return float(d.get("rho", 0.0)), u[:dim], float(d["p"])


def _xyz(v, dim):
    v = [float(a) for a in v] + [0.0, 0.0, 0.0]
    return np.array(v[:dim])


def initial_field(ic: dict, dim: int, gamma: float):
    """The reference's initial condition as a function of the node
    coordinates (dim, n) -> primitive (rho, u, v, [w], p)."""
    kind = ic.get("type")
    if kind == "constant":
        rho, u, p = _prim_state(ic, dim)

        def f(X):
            one = np.ones(X.shape[1])
            return [rho * one] + [ui * one for ui in u] + [p * one]
        return f
    if kind in ("planeBreakup", "sphericalBreakup"):
        o = _xyz(ic["origin"], dim)
        left, right = _prim_state(ic["left"], dim), _prim_state(ic["right"], dim)
        v1 = [left[0], *left[1], left[2]]
        v2 = [right[0], *right[1], right[2]]
        if kind == "planeBreakup":  # ICPlaneBreakup: n . (x - origin) < 0 -> left
            nrm = _xyz(ic["normal"], dim)

            def f(X):
                side = (nrm[:, None] * (X - o[:, None])).sum(0) < 0
                return [np.where(side, a, b) for a, b in zip(v1, v2)]
            return f
        r2 = float(ic["radius"]) ** 2
        r2d = 0.2 * 0.2 * r2

        def f(X):
            # ICSphericalBreakup: inside -> left; a band r^2 - R^2 < 0.04 R^2 on
            # the ramp from R to 1.2 R (cut where the band ends); else right
            d2 = ((X - o[:, None]) ** 2).sum(0)
            s = d2 - r2
            r1, rr = np.sqrt(r2), np.sqrt(r2) + np.sqrt(r2d)
            dist = np.sqrt(d2)
            out = []
            for a, b in zip(v1, v2):
                ramp = (dist - r1) * (b - a) / (rr - r1) + a
                out.append(np.where(s < 0, a, np.where(s < r2d, ramp, b)))
            return out
        return f
    if kind == "densityPulse":
        o = _xyz(ic["origin"], dim)
        eps = float(ic["epsilon"])
        u = [float(v) for v in ic["U"]] + [0.0, 0.0, 0.0]
        p = float(ic["p"])
        pi_ref = 3.14169265  # the constant ICDensityPulse uses for pi

        def f(X):
            r2m1 = ((X - o[:, None]) ** 2).sum(0) - 1.0
            rho = (1.0 - (gamma - 1.0) * eps * eps * np.exp(r2m1) /
                   (8.0 * gamma * pi_ref * pi_ref)) ** (1.0 / (gamma - 1.0))
            one = np.ones(X.shape[1])
            return [rho] + [ui * one for ui in u[:dim]] + [p * one]
        return f
    raise CaseError(f"unknown initial condition type {kind!r}")


# ---- the case -----------------------------------------------------------------

_RS = {"Rusanov": RS_RUSANOV, "LLF": RS_LLF, "HLL": RS_HLL, "HLLC": RS_HLLC}
_IND = {"Nowhere": IND_NOWHERE, "Everywhere": IND_EVERYWHERE, "BJ": IND_BJ, "Shu": IND_SHU}
_LIM = {"FinDiff": LIM_FINDIFF, "Multi": LIM_MULTI}


def _bc(patch: dict, dim: int, gamma: float):
    """One boundaryField entry -> (RKDG_BC_* code, state) as the reference's
    integrator factory builds it (case_manager.cpp:700-800)."""
    t = patch.get("type")
    if t == "slip":
        return BC_SLIP, None
    if t == "outlet":
        return BC_OPEN, None
    if t == "supersonicInlet":
        rho = float(patch["rhoI"])
        u = [float(v) for v in patch["UI"]] + [0.0, 0.0, 0.0]
        p = float(patch["pI"])
        # the reference's inlet energy omits the third velocity component
        E = p / (gamma - 1.0) + 0.5 * rho * (u[0] * u[0] + u[1] * u[1])
        return BC_SUPERSONIC_INLET, [rho] + [rho * v for v in u[:dim]] + [E]
    if t == "subsonicInletTotalPressure":
        return BC_SUBSONIC_INLET_TOTAL_PRESSURE, [float(patch["pTot"]), float(patch["TTot"])]
    if t == "subsonicInletFixedPressure":
        return BC_SUBSONIC_INLET_FIXED_PRESSURE, [float(patch["pFix"]), float(patch["TTot"])]
    if t == "totalPressureFixedTemperatureOutlet":
        return BC_TOTAL_PRESSURE_OUTLET, [float(patch["pTot"]), float(patch["TFix"])]
    if t == "fixedPressureOutlet":
        return BC_FIXED_PRESSURE_OUTLET, [float(patch["pFix"])]
    if t == "charOutlet":
        # case_manager.cpp:779-802: rho, rho u, rho v, rho w, then the energy
        # without the third velocity component (in 2D it overwrites rho w)
        rho = float(patch["rhoI"])
        u = [float(v) for v in patch["UI"]] + [0.0, 0.0]
        p = float(patch["pI"])
        E = p / (gamma - 1.0) + 0.5 * rho * (u[0] * u[0] + u[1] * u[1])
        return BC_CHAR_OUTLET, [rho] + [rho * v for v in u[:dim]] + [E]
    raise CaseError(f"unknown boundary condition type {t!r} (the reference exits here)")


def load_case(case_dir: str, settings: dict | None = None) -> C.Case:
    """Build the case of a reference case directory (settings.yml and the
    Gmsh v2.2 mesh it names, relative to the directory)."""
    s = settings if settings is not None else read_settings(os.path.join(case_dir, "settings.yml"))
    ms = s["mesh"]
    if int(ms.get("adaptive", 0)):
        raise CaseError("adaptive cases need the reference's error estimator (MFEM); "
                        "refine with mesh.refine_nc and Context.update_mesh instead")
    path = os.path.join(case_dir, str(ms["file"]))
    mesh = M.read_gmsh22(path)
    names = M.read_gmsh22_physical_names(path)
    for _ in range(int(ms.get("serialRefLevels", 0))):  # Mesh::UniformRefinement
        if mesh.geom == M.GEOM_TRIANGLE:
            raise CaseError("uniform refinement of triangle meshes is not supported")
        mesh = M.refine_nc(mesh, range(mesh.num_elements))
    dim = mesh.dim
    ph = s["physics"]
    gamma = float(ph.get("gamma", 1.4))
    covolume = float(ph["covolume"]) if ph.get("type") == "covolume" else 0.0
    R = float(ph.get("R", 1.0))
    sp = s["spatial"]
    rsn = sp["riemannSolver"]
    if rsn not in _RS:
        raise CaseError(f"unknown Riemann solver type {rsn!r}")
    lim = sp["limiter"]
    if lim.get("indicator") not in _IND:
        raise CaseError(f"unknown indicator type {lim.get('indicator')!r}")
    if lim.get("type") not in _LIM:
        raise CaseError(f"unknown limiter type {lim.get('type')!r}")
    quirks = LIMITER_LINEARIZE if int(lim.get("linearize", 0)) else 0
    limiter = (_LIM[lim["type"]], _IND[lim["indicator"]], FUN_MICHALAK,
               int(lim.get("haveLastHope", 1)), quirks)
    bcs = []
    for name, patch in (s.get("boundaryField") or {}).items():
        hit = names.get(name)
        if hit is None or hit[0] != dim - 1:
            continue  # "No geometric group for boundary": the reference skips it
        code, state = _bc(patch, dim, gamma)
        bcs.append((hit[1], code, state))
    tm = s["time"]
    order = int(tm.get("order", 0))
    tableau = {2: TABLEAU_REFERENCE_RK2, 3: TABLEAU_REFERENCE_RK3}.get(order)
    if tableau is None:
        raise CaseError(f"time order {order} (the reference knows 2 and 3)")
    fixed = tm.get("type") == "constant"
    return C.Case(os.path.basename(os.path.normpath(case_dir)), mesh, int(sp["polyOrder"]),
                  _RS[rsn], AVG_TRRS, gamma=gamma, covolume=covolume, bcs=bcs, limiter=limiter,
                  tableau=tableau, t_end=float(tm["tEnd"]),
                  cfl=-1.0 if fixed else float(tm["CoMax"]), dt_mode=2 if fixed else 0,
                  dt0=float(tm.get("dt", 0.0)),
                  ic=initial_field(s["internalField"], dim, gamma), gas_constant=R)


# ---- running and output --------------------------------------------------------

RESTART_FIELD = "restart_conservative_vars"
_FRAME = re.compile(r"^restart_(\d{6,})$")


def restart_name(cycle: int) -> str:
    return f"restart_{cycle:06d}"


def save_restart(out_dir: str, cycle: int, t: float, dt: float, mesh: M.Mesh, order: int,
                 x) -> str:
    """Write restart frame ``cycle`` (the reference's restart_dc.Save with
    SetCycle / SetTime / SetTimeStep, main.cpp:757-760): the directory
    ``restart_<cycle>`` with the mesh and the conservative state (MFEM byNODES
    order) and the root ``restart_<cycle>.json`` with cycle, time and time
    step.  Returns the frame's name."""
    name = restart_name(cycle)
    d = os.path.join(out_dir, name)
    os.makedirs(d, exist_ok=True)
    m = mesh.contiguous()
    np.savez(os.path.join(d, "mesh.npz"), dim=m.dim, geom=m.geom, elem_vertices=m.elem_vertices,
             elem_coords=m.elem_coords, bdr_vertices=m.bdr_vertices, bdr_attr=m.bdr_attr)
    xs = x.detach().cpu().numpy() if hasattr(x, "detach") else np.asarray(x)
    np.save(os.path.join(d, RESTART_FIELD + ".npy"), np.ascontiguousarray(xs, dtype=np.float64))
    root = {"cycle": int(cycle), "time": float(t), "time_step": float(dt), "order": int(order),
            "mesh": f"{name}/mesh.npz", "fields": {RESTART_FIELD: f"{name}/{RESTART_FIELD}.npy"}}
    with open(os.path.join(out_dir, name + ".json"), "w") as fh:
        json.dump(root, fh, indent=1)
    return name


def load_restart(out_dir: str, cycle: int) -> dict:
    """Read restart frame ``cycle`` (restart_data_c.Load(restartCycle),
    case_manager.cpp:237-260, 488-505): mesh, order, state, time, cycle and
    time step.  A missing frame or field is a CaseError, as the reference
    prints and exits."""
    name = restart_name(cycle)
    rp = os.path.join(out_dir, name + ".json")
    if not os.path.isfile(rp):
        raise CaseError(f"Error loading data collection: no restart frame {name} in {out_dir}")
    with open(rp) as fh:
        root = json.load(fh)
    if RESTART_FIELD not in root.get("fields", {}):
        raise CaseError(f"The given data collection has no '{RESTART_FIELD}' field.")
    z = np.load(os.path.join(out_dir, root["mesh"]))
    mesh = M.Mesh(int(z["dim"]), int(z["geom"]), z["elem_vertices"], z["elem_coords"],
                  z["bdr_vertices"], z["bdr_attr"])
    x = np.load(os.path.join(out_dir, root["fields"][RESTART_FIELD]))
    return {"mesh": mesh, "order": int(root["order"]), "x": x, "time": float(root["time"]),
            "cycle": int(root["cycle"]), "time_step": float(root["time_step"])}


class RestartFrames:
    """The reference's queue of saved frames (initializeRestartQueue and
    cleanPreviousRestartFrames, case_manager.cpp:895-985): frames already in
    the directory join the queue, those of a later cycle than the one a run
    restarts from are removed; after each save the oldest frames beyond
    ``n_saved`` are removed.  Only names of the form restart_<digits> (and
    their roots) are touched."""

    def __init__(self, out_dir: str, n_saved: int, restart_cycle: int | None = None):
        self.out_dir, self.n_saved = out_dir, int(n_saved)
        current = restart_name(restart_cycle if restart_cycle is not None else 0)
        self.queue: list[str] = []
        for entry in sorted(os.listdir(out_dir)):
            if not (_FRAME.match(entry) and os.path.isdir(os.path.join(out_dir, entry))):
                continue
            if entry > current:
                self._remove(entry)
            else:
                self.queue.append(entry)
        if not self.queue:
            self.queue.append(restart_name(0))

    def _remove(self, name: str) -> None:
        shutil.rmtree(os.path.join(self.out_dir, name), ignore_errors=True)
        root = os.path.join(self.out_dir, name + ".json")
        if os.path.isfile(root):
            os.remove(root)

    def saved(self, cycle: int) -> None:
        self.queue.append(restart_name(cycle))
        self.queue.sort()
        if len(self.queue) > self.n_saved:
            self._remove(self.queue.pop(0))


def run_case(case_dir: str, device: int = 0, precision: int = 0, max_steps: int = 0,
             t_end: float | None = None, settings: dict | None = None,
             out_dir: str | None = None, restart_frames: bool = False):
    """Run a case directory on the GPU with the reference's time bookkeeping;
    returns (case, context, final state as a CUDA tensor, run info).

    The initial state is the projected initial field, limited (main.cpp:
    264-265), or with ``time.restart`` set the state of restart frame
    ``time.restartCycle`` in ``out_dir`` (default: the case directory), also
    limited, continuing from that frame's time, cycle and time step.  With
    ``restart_frames`` (or a restart) frames are written as the reference
    writes them: one before the loop (cycle 0 and time 0, also when the run
    restarts), every ``postProcess.visSteps`` steps and at the end, keeping
    the ``time.nSavedFrames`` newest.  The run stops at tEnd (or t_end, or
    after max_steps steps)."""
    import torch

    from .solver import Context
    s = settings if settings is not None else read_settings(os.path.join(case_dir, "settings.yml"))
    case = load_case(case_dir, s)
    out_dir = case_dir if out_dir is None else out_dir
    tm = s.get("time", {})
    restart = bool(tm.get("restart", False))
    write = restart_frames or restart
    vis_steps = max(1, int((s.get("postProcess") or {}).get("visSteps", 1)))
    t_stop = case.t_end if t_end is None else t_end
    t0, ti, dt = 0.0, 0, None
    if restart:
        fr = load_restart(out_dir, int(tm.get("restartCycle", 0)))
        if fr["order"] != case.order:
            raise CaseError("the restart frame's polynomial order differs from the settings'")
        case.mesh = fr["mesh"]
        t0, ti, dt = fr["time"], fr["cycle"], fr["time_step"]
    ctx = Context(case.mesh, case.order, device=device, precision=precision)
    C.configure_context(case, ctx)
    if restart:
        x = torch.tensor(fr["x"], dtype=torch.float64, device=f"cuda:{device}")
        if x.numel() != ctx.n:
            raise CaseError("the restart frame's state does not match its mesh")
    else:
        x = torch.tensor(C.project(case, ctx.node_coords()), dtype=torch.float64,
                         device=f"cuda:{device}")
    if not write:
        info = ctx.run(x, t_stop, cfl=case.cfl, dt0=case.dt0, dt_mode=case.dt_mode,
                       max_steps=max_steps)
        return case, ctx, x, info
    frames = RestartFrames(out_dir, int(tm.get("nSavedFrames", 0)),
                           ti if restart else None)
    ctx.limit(x)  # l->update(sol) after loadInitialSolution (main.cpp:264-265)
    if dt is None:  # the initial dt of main.cpp:467-484 (as rkdg_run forms it)
        dt = case.dt0 if case.dt_mode == 2 else \
            case.cfl * ctx.hmin() / ctx.face_speed(x) / (2 * case.order + 1)
    save_restart(out_dir, 0, 0.0, dt, case.mesh, case.order, x)  # main.cpp:492-495
    t, steps, sum_dt, done = t0, 0, 0.0, False
    while not done:
        chunk = vis_steps - (ti % vis_steps)
        if max_steps > 0:
            chunk = min(chunk, max_steps - steps)
        info = ctx.run_continue(x, t, dt, t_stop, cfl=case.cfl, dt_mode=case.dt_mode,
                                max_steps=chunk)
        t, dt = info["t"], info["dt"]
        ti += info["steps"]
        steps += info["steps"]
        sum_dt += info["sum_dt"]
        done = t >= t_stop - 1e-8 * dt
        if done or ti % vis_steps == 0:
            save_restart(out_dir, ti, t, dt, case.mesh, case.order, x)
            frames.saved(ti)
        if max_steps > 0 and steps >= max_steps:
            break
    return case, ctx, x, {"steps": steps, "t": t, "dt": dt, "sum_dt": sum_dt, "cycle": ti}


_VTK_CELL = {M.GEOM_TRIANGLE: 5, M.GEOM_SQUARE: 9, M.GEOM_CUBE: 12}


def write_vtu(path: str, mesh: M.Mesh, means: np.ndarray, gamma: float = 1.4,
              covolume: float = 0.0) -> None:
    """ParaView file (VTK XML unstructured grid, ASCII) of the cell means
    means[neq][ne] of a state: density, velocity, pressure and energy per
    cell on the elements' corners (MFEM vertex orders are VTK's for
    triangles, quadrilaterals and hexahedra)."""
    ne, nv = mesh.elem_vertices.shape
    dim = mesh.dim
    m = np.asarray(means, np.float64).reshape(dim + 2, ne)
    rho, mom, E = m[0], m[1:1 + dim], m[dim + 1]
    vel = mom / rho
    p = (gamma - 1.0) * (E - 0.5 * (mom * vel).sum(0)) / (1.0 - covolume * rho)
    pts = np.zeros((ne * nv, 3))
    pts[:, :dim] = mesh.elem_coords.reshape(-1, dim)
    v3 = np.zeros((ne, 3))
    v3[:, :dim] = vel.T

    def arr(a):
        return " ".join(repr(float(v)) for v in np.ravel(a))

    with open(path, "w") as fh:
        fh.write('<?xml version="1.0"?>\n<VTKFile type="UnstructuredGrid" version="0.1" '
                 'byte_order="LittleEndian">\n<UnstructuredGrid>\n')
        fh.write(f'<Piece NumberOfPoints="{ne * nv}" NumberOfCells="{ne}">\n')
        fh.write('<Points><DataArray type="Float64" NumberOfComponents="3" format="ascii">'
                 f"{arr(pts)}</DataArray></Points>\n<Cells>\n")
        fh.write('<DataArray type="Int64" Name="connectivity" format="ascii">'
                 f'{" ".join(str(i) for i in range(ne * nv))}</DataArray>\n')
        fh.write('<DataArray type="Int64" Name="offsets" format="ascii">'
                 f'{" ".join(str(nv * (e + 1)) for e in range(ne))}</DataArray>\n')
        fh.write('<DataArray type="UInt8" Name="types" format="ascii">'
                 f'{" ".join([str(_VTK_CELL[mesh.geom])] * ne)}</DataArray>\n</Cells>\n')
        fh.write('<CellData Scalars="rho">\n')
        fh.write(f'<DataArray type="Float64" Name="rho" format="ascii">{arr(rho)}</DataArray>\n')
        fh.write('<DataArray type="Float64" Name="U" NumberOfComponents="3" format="ascii">'
                 f"{arr(v3)}</DataArray>\n")
        fh.write(f'<DataArray type="Float64" Name="p" format="ascii">{arr(p)}</DataArray>\n')
        fh.write(f'<DataArray type="Float64" Name="E" format="ascii">{arr(E)}</DataArray>\n')
        fh.write("</CellData>\n</Piece>\n</UnstructuredGrid>\n</VTKFile>\n")
