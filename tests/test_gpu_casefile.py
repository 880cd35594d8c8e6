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
