"""A case directory (settings.yml + Gmsh v2.2 mesh) run end to end on the GPU
through rkdg3d_gb300.casefile.run_case, against the oracle running the same
case; plus the ParaView output of the result."""
import pytest
import torch

from oracle.refcpu import Oracle
from rkdg3d_gb300 import cases
from rkdg3d_gb300 import casefile as CF
from tests.helpers import rel_l1
from tests.test_casefile import tube  # noqa: F401  (fixture)

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("refine", [0, 1])
def test_run_case_against_oracle(cuda, tube, refine, tmp_path):  # noqa: F811
    s = CF.read_settings(f"{tube}/settings.yml")
    s["mesh"]["serialRefLevels"] = refine
    case, ctx, x, info = CF.run_case(tube, settings=s)
    assert info["steps"] > 5
    orc = Oracle(case.mesh, case.order)
    cases.configure_oracle(case, orc)
    x_ref, info_ref = orc.run(cases.project(case, orc.node_coords()), case.t_end, cfl=case.cfl,
                              dt0=case.dt0, dt_mode=case.dt_mode)
    assert info["steps"] == info_ref["steps"]
    # a limited run: indicator switches part the paths by ~1e-10 (see the limiter tests)
    assert rel_l1(x.cpu().numpy(), x_ref) < 1e-8
    md = torch.empty(ctx.neq * ctx.ne, dtype=torch.float64, device="cuda")
    ctx.cell_means(x, md)
    path = str(tmp_path / "tube.vtu")
    CF.write_vtu(path, case.mesh, md.cpu().numpy().reshape(ctx.neq, ctx.ne))
    assert open(path).read().count("<DataArray") == 8  # points, 3 cell arrays, 4 fields


def test_run_case_restart_frames(cuda, tube, tmp_path):  # noqa: F811
    """Frames written every visSteps steps hold the state an uninterrupted
    run has at that cycle (bit for bit); a restart continues from a frame's
    time, cycle and dt after limiting the loaded state, as the reference
    does."""
    s = CF.read_settings(f"{tube}/settings.yml")
    s["postProcess"] = {"visSteps": 5}
    s["time"]["nSavedFrames"] = 3
    out = str(tmp_path / "run")
    import os
    os.makedirs(out)
    case, ctx, x, info = CF.run_case(tube, settings=s, out_dir=out, restart_frames=True)
    n = info["steps"]
    assert n > 10 and info["cycle"] == n
    saved = sorted(e for e in os.listdir(out) if e.startswith("restart_") and e[8:].isdigit())
    assert len(saved) == 3 and saved[-1] == CF.restart_name(n)
    # the final frame is the uninterrupted run's final state
    _, _, x1, info1 = CF.run_case(tube, settings=s)
    assert info1["steps"] == n and torch.equal(x, x1)
    fr = CF.load_restart(out, n)
    assert (torch.tensor(fr["x"]) == x.cpu()).all() and fr["time"] == info1["t"]
    # a frame in the middle: the uninterrupted run stopped at that cycle
    mid = int(saved[-2][8:])
    _, _, x2, info2 = CF.run_case(tube, settings=s, max_steps=mid)
    fm = CF.load_restart(out, mid)
    assert (torch.tensor(fm["x"]) == x2.cpu()).all()
    assert fm["time"] == info2["t"] and fm["time_step"] == info2["dt"]
    # restart from it: limit the frame's state, continue with its t and dt
    s2 = CF.read_settings(f"{tube}/settings.yml")
    s2["postProcess"] = {"visSteps": 5}
    s2["time"].update({"restart": True, "restartCycle": mid, "nSavedFrames": 3})
    _, ctx3, x3, info3 = CF.run_case(tube, settings=s2, out_dir=out)
    xr = torch.tensor(fm["x"], dtype=torch.float64, device="cuda")
    ctx3.limit(xr)
    ref = ctx3.run_continue(xr, fm["time"], fm["time_step"], case.t_end, cfl=case.cfl,
                            dt_mode=case.dt_mode)
    assert torch.equal(x3, xr) and info3["cycle"] == mid + ref["steps"]
    assert info3["t"] == ref["t"]
    # frames later than the restarted cycle were removed before the run wrote
    # its own; frame 0 holds the restarted state with time 0, as the reference
    # writes it before its loop
    f0 = CF.load_restart(out, 0)
    assert f0["time"] == 0.0 and f0["cycle"] == 0
