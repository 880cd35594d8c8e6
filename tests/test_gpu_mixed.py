"""FP32-bulk path: error against the plain FP64 path (which is itself
parity-checked against the oracle).  Target from the precision study:
relative L1 density error <= 1e-6."""
import numpy as np
import pytest
import torch

from rkdg3d_gb300 import cases
from rkdg3d_gb300 import mesh as M
from rkdg3d_gb300.solver import FP32_BULK, FP64, RS_HLLC, RS_RUSANOV, Context
from tests.helpers import periodic_case, random_state, rel_l1

pytestmark = pytest.mark.gpu


def make(case, prec):
    ctx = Context(case.mesh, case.order, device=0, precision=prec)
    cases.configure_context(case, ctx)
    return ctx


@pytest.mark.parametrize("variant", [0, 2, 3, 4, 5, 6])
def test_mixed_rhs_close_to_fp64(cuda, variant):
    """FP32-bulk right-hand side (fused team kernel, or face pass + element
    pass) against the plain FP64 one."""
    from rkdg3d_gb300.solver import TUNE_HEX_KERNEL
    case = cases.pulse3d(n=6, order=2, steps=10)
    c64, c32 = make(case, FP64), make(case, FP32_BULK)
    c32.set_tuning(TUNE_HEX_KERNEL, variant)
    x = torch.tensor(random_state(c64.node_coords(), seed=9, amp=0.05, vel=0.1), device="cuda",
                     dtype=torch.float64)
    y64 = torch.empty_like(x)
    y32 = torch.empty_like(x)
    m64 = c64.rhs(x, y64)
    m32 = c32.rhs(x, y32)
    assert rel_l1(y32.cpu().numpy(), y64.cpu().numpy()) < 1e-5
    assert abs(m32 - m64) < 1e-5 * m64


def test_mixed_pulse_density_error(cuda):
    """Acoustic pulse (C2 set-up at 16^3): FP32-bulk vs FP64 after 100 steps."""
    case = cases.pulse3d(n=16, order=2, steps=100)
    c64, c32 = make(case, FP64), make(case, FP32_BULK)
    x0 = torch.tensor(cases.project(case, c64.node_coords()), device="cuda", dtype=torch.float64)
    dt = case.cfl * c64.hmin() / c64.face_speed(x0) / 5.0
    a, b = x0.clone(), x0.clone()
    c64.run(a, 1e30, dt0=dt, dt_mode=2, max_steps=100)
    c32.run(b, 1e30, dt0=dt, dt_mode=2, max_steps=100)
    nd = c64.ndofs
    ra, rb = a.cpu().numpy()[:nd], b.cpu().numpy()[:nd]
    err = rel_l1(rb, ra)
    assert err < 1e-6, err
    # the pulse has moved: the comparison is not trivially between initial states
    assert rel_l1(ra, x0.cpu().numpy()[:nd]) > 1e-5


def test_mixed_sod_limited_close(cuda):
    case = cases.sod(nx=80, ny=2, t_end=0.05)
    c64, c32 = make(case, FP64), make(case, FP32_BULK)
    x0 = cases.project(case, c64.node_coords())
    a = torch.tensor(x0, device="cuda", dtype=torch.float64)
    b = a.clone()
    c64.run(a, case.t_end, case.cfl)
    c32.run(b, case.t_end, case.cfl)
    nd = c64.ndofs
    assert rel_l1(b.cpu().numpy()[:nd], a.cpu().numpy()[:nd]) < 1e-4


def test_mixed_conservation_periodic(cuda):
    case = periodic_case(M.GEOM_CUBE, 4, 2, RS_HLLC)
    ctx = make(case, FP32_BULK)
    x = torch.tensor(random_state(ctx.node_coords(), seed=3, amp=0.1, vel=0.2), device="cuda",
                     dtype=torch.float64)
    t0 = ctx.totals(x)
    for _ in range(10):
        ctx.step(x, 2e-3)
    t1 = ctx.totals(x)
    assert np.all(np.abs(t1 - t0) <= 1e-9 * np.abs(t0).max())


def test_mixed_autotune_small_elements(cuda):
    """FP32-bulk Q1 quadrilaterals: the autotuner keeps the CTA sizes within
    the 128 threads the FP32 kernels of small elements are built for, and the
    right-hand side stays within the FP32-bulk bound of FP64."""
    from tests.helpers import walled_case
    from rkdg3d_gb300.solver import BC_SLIP, FUN_MICHALAK, IND_BJ, LIM_MULTI, RS_HLLC as HLLC
    case = walled_case(M.GEOM_SQUARE, 12, 1, HLLC, bc=BC_SLIP)
    case.limiter = (LIM_MULTI, IND_BJ, FUN_MICHALAK, 1, 0)
    c64, c32 = make(case, FP64), make(case, FP32_BULK)
    x = torch.tensor(random_state(c64.node_coords(), seed=2, amp=0.05, vel=0.1), device="cuda",
                     dtype=torch.float64)
    choice = c32.autotune(x)
    assert choice["generic_block"] in (64, 128) and choice["limiter_block"] in (64, 128)
    y64, y32 = torch.empty_like(x), torch.empty_like(x)
    c64.rhs(x, y64)
    c32.rhs(x, y32)
    assert rel_l1(y32.cpu().numpy(), y64.cpu().numpy()) < 1e-5
