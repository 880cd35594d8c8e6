"""Tensor-core variant of the face-once tile kernel (hexahedral kernel 6):
the Q2 volume contraction as TF32 MMAs (tcgen05) with split hi/lo operands.

Against the same kernel's FP32 sweeps (variant 5) the right-hand sides agree
to the split's accuracy (about 2^-21 per product), and against the plain
FP64 path within the FP32-bulk bounds of the other kernels."""
import numpy as np
import pytest
import torch

from rkdg3d_gb300 import cases
from rkdg3d_gb300 import mesh as M
from rkdg3d_gb300.solver import (AVG_EINFELDT, BC_SLIP, FP32_BULK, FP64, RS_HLLC, RS_LLF,
                                 TUNE_HEX_KERNEL, Context)
from tests.helpers import periodic_case, random_state, rel_l1, walled_case

pytestmark = pytest.mark.gpu


def make(case, prec, variant=0):
    ctx = Context(case.mesh, case.order, device=0, precision=prec)
    cases.configure_context(case, ctx)
    if variant:
        ctx.set_tuning(TUNE_HEX_KERNEL, variant)
    return ctx


CASES = {
    "periodic-6": lambda: periodic_case(M.GEOM_CUBE, 6, 2, RS_LLF),
    "walls-5": lambda: walled_case(M.GEOM_CUBE, 5, 2, RS_HLLC, AVG_EINFELDT, bc=BC_SLIP),
    "pulse-8": lambda: cases.pulse3d(n=8, order=2, steps=10),
}


@pytest.mark.parametrize("name", list(CASES))
def test_tc_rhs_against_sweeps_and_fp64(cuda, name):
    case = CASES[name]()
    c64, c5, c6 = make(case, FP64), make(case, FP32_BULK, 5), make(case, FP32_BULK, 6)
    x = torch.tensor(random_state(c64.node_coords(), seed=11, amp=0.05, vel=0.1), device="cuda",
                     dtype=torch.float64)
    y64, y5, y6 = (torch.empty_like(x) for _ in range(3))
    m64 = c64.rhs(x, y64)
    m5 = c5.rhs(x, y5)
    m6 = c6.rhs(x, y6)
    a64, a5, a6 = (y.cpu().numpy() for y in (y64, y5, y6))
    assert np.all(np.isfinite(a6))
    assert not np.array_equal(a6, a5)  # the tensor-core kernel ran (it rounds differently)
    assert rel_l1(a6, a5) < 3e-6, rel_l1(a6, a5)
    assert rel_l1(a6, a64) < 1e-5, rel_l1(a6, a64)
    assert m6 == m5  # the wave speeds do not go through the tensor cores
    assert abs(m6 - m64) < 1e-5 * m64


def test_tc_pulse_run_density_error(cuda):
    """C2's set-up at 16^3, 100 steps: the tensor-core kernel's density
    against the FP64 path, as the FP32-bulk bound of the sweep kernel."""
    case = cases.pulse3d(n=16, order=2, steps=100)
    c64, c6 = make(case, FP64), make(case, FP32_BULK, 6)
    x0 = torch.tensor(cases.project(case, c64.node_coords()), device="cuda", dtype=torch.float64)
    dt = case.cfl * c64.hmin() / c64.face_speed(x0) / 5.0
    a, b = x0.clone(), x0.clone()
    c64.run(a, 1e30, dt0=dt, dt_mode=2, max_steps=100)
    c6.run(b, 1e30, dt0=dt, dt_mode=2, max_steps=100)
    nd = c64.ndofs
    err = rel_l1(b.cpu().numpy()[:nd], a.cpu().numpy()[:nd])
    assert err < 1e-6, err
