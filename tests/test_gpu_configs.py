"""The benchmark configurations at their own sizes against the oracle (FP64
device path through the C ABI).

  C1  Sod 200x4 Q1, HLLC + Einfeldt, BJ limiter, SSP-RK3 CFL 0.3, t = 0.2:
      the whole run, initial limit included (main.cpp:264-265);
  C3  double Mach reflection on the 524,288 jittered P1 triangles, HLL +
      TRRS, Venkatakrishnan: initial limit, right-hand side and one step
      <= 1e-12, then a bounded run;
  C2  the 64^3 Q2 hexahedral pulse: one right-hand side <= 1e-12.

Limited runs amplify round-off through the limiter's hard switches (the
+-1e-3 indicator thresholds, stencil min/max), so a limited run is bounded by
how far the oracle moves from itself under a 1e-15 relative perturbation of
its input, with the step count and the dt bookkeeping exact.
"""
import numpy as np
import pytest
import torch

from oracle.refcpu import Oracle, OracleError
from rkdg3d_gb300 import cases
from rkdg3d_gb300.solver import (FP32_BULK, FUN_BJ, FUN_MICHALAK, TABLEAU_REFERENCE_RK3, Context,
                                 UnphysicalStateError)
from tests.helpers import rel_l1

pytestmark = pytest.mark.gpu


def pair(case, precision=0):
    ctx = Context(case.mesh, case.order, device=0, precision=precision)
    cases.configure_context(case, ctx)
    orc = Oracle(case.mesh, case.order)
    cases.configure_oracle(case, orc)
    return ctx, orc


def dev(x):
    return torch.tensor(x, dtype=torch.float64, device="cuda:0")


def _limited_run_check(ctx, orc, case, max_steps=0):
    x0 = cases.project(case, orc.node_coords())
    x_ref, info_ref = orc.run(x0, case.t_end, case.cfl, max_steps=max_steps)
    rng = np.random.default_rng(0)
    x_pert, _ = orc.run(x0 * (1 + 1e-15 * rng.uniform(-1, 1, x0.size)), case.t_end, case.cfl,
                        max_steps=max_steps)
    xd = dev(x0)
    info = ctx.run(xd, case.t_end, case.cfl, max_steps=max_steps)
    assert info["steps"] == info_ref["steps"]
    # the booked time ends with the dt of the final state's wave speed
    # (t += new dt, main.cpp:701), which moves with the limited state
    assert info["t"] == pytest.approx(info_ref["t"], rel=1e-3)
    nd = orc.ndofs
    rho = xd.cpu().numpy()[:nd]
    d_gpu = rel_l1(rho, x_ref[:nd])
    d_self = rel_l1(x_pert[:nd], x_ref[:nd])
    return d_gpu, d_self, info


@pytest.mark.parametrize("function,tableau", [(FUN_BJ, None), (FUN_MICHALAK, TABLEAU_REFERENCE_RK3)],
                         ids=["bj-sspRK3", "shipped-michalak-referenceRK3"])
def test_c1_sod_full_run(cuda, function, tableau):
    """C1 exactly: 200x4 quads, t_end = 0.2 (and the reference as shipped:
    its "BJ" indicator is Michalak, its order-3 arrays give a21=0, a31=1)."""
    kw = {"function": function}
    if tableau is not None:
        kw["tableau"] = tableau
    case = cases.sod(**kw)
    assert case.mesh.num_elements == 800 and case.t_end == 0.2
    ctx, orc = pair(case)
    d_gpu, d_self, info = _limited_run_check(ctx, orc, case)
    assert info["steps"] > 500
    assert d_gpu < 1e-3
    # over 500+ limited steps FP64 rounding differences (device FMA
    # contraction against the oracle's separate products) grow to ~1e-11
    assert d_gpu < 10 * d_self + 1e-10, (d_gpu, d_self)


def test_initial_limit_is_part_of_the_run(cuda):
    """rkdg_run limits the projected state before its first dt, as the
    reference does; with limit_initial=False it steps the state as given."""
    case = cases.sod(nx=45, ny=2, t_end=0.02)  # the jump lies inside element 22
    ctx, orc = pair(case)
    x0 = cases.project(case, orc.node_coords())
    a, b = dev(x0), dev(x0)
    ctx.run(a, case.t_end, case.cfl)
    ctx.limit(b)
    ctx.run(b, case.t_end, case.cfl, limit_initial=False)
    assert torch.equal(a, b)
    xr, _ = orc.run(x0, case.t_end, case.cfl)
    assert rel_l1(a.cpu().numpy(), xr) < 1e-10  # limited steps amplify FP64 rounding
    # the unlimited projection of the jump: the device and the oracle stop on
    # the same non-physical state, or agree
    c = dev(x0)
    gpu_err = orc_err = None
    try:
        ctx.run(c, case.t_end, case.cfl, limit_initial=False)
    except UnphysicalStateError as ex:
        gpu_err = ex
    try:
        xr2, _ = orc.run(x0, case.t_end, case.cfl, limit_initial=False)
    except OracleError as ex:
        orc_err = ex
    assert (gpu_err is None) == (orc_err is None), (gpu_err, orc_err)
    if gpu_err is None:
        assert not torch.equal(a, c)
        assert rel_l1(c.cpu().numpy(), xr2) < 1e-10


@pytest.fixture(scope="module")
def dmr():
    case = cases.double_mach()
    assert case.mesh.num_elements == 524288
    ctx, orc = pair(case)
    x0 = cases.project(case, orc.node_coords())
    return case, ctx, orc, x0


def test_c3_full_mesh_limit_rhs_step(cuda, dmr):
    case, ctx, orc, x0 = dmr
    xl_ref = orc.limit(x0)
    xd = dev(x0)
    ctx.limit(xd)
    xl = xd.cpu().numpy()
    assert rel_l1(xl, xl_ref) < 1e-12
    y_ref, m_ref = orc.rhs(xl_ref)
    yd = torch.empty_like(xd)
    m = ctx.rhs(dev(xl_ref), yd)
    assert rel_l1(yd.cpu().numpy(), y_ref) < 1e-12
    assert m == pytest.approx(m_ref, rel=1e-12)
    dt = case.cfl * orc.hmin() / orc.face_speed(xl_ref) / (2 * case.order + 1)
    xs_ref, _ = orc.step(xl_ref, dt)
    xs = dev(xl_ref)
    ctx.step(xs, dt)
    assert rel_l1(xs.cpu().numpy(), xs_ref) < 1e-12


def test_c3_full_mesh_bounded_run(cuda, dmr):
    """The first 20 steps of C3 (initial limit, CFL dt each step)."""
    case, ctx, orc, _ = dmr
    d_gpu, d_self, info = _limited_run_check(ctx, orc, case, max_steps=20)
    assert info["steps"] == 20
    assert d_gpu < 1e-8
    assert d_gpu < 10 * d_self + 1e-12, (d_gpu, d_self)


def test_c2_rhs_64cubed(cuda):
    """C2 at its own size: 64^3 periodic Q2 hexahedra, one right-hand side
    of the projected pulse, FP64 device path <= 1e-12 against the oracle; the
    FP32-bulk path's error against it is reported by the same comparison."""
    case = cases.pulse3d(n=64)
    ctx, orc = pair(case)
    x0 = cases.project(case, orc.node_coords())
    # the pulse's right-hand side is small against the state: test the
    # perturbation part (rho - 1) of a moving state too
    rng = np.random.default_rng(5)
    nd = orc.ndofs
    x = x0.copy()
    x[nd:4 * nd] = 0.01 * np.sin(2 * np.pi * rng.uniform(size=3 * nd))
    # the pulse at rest: outside the pulse (most of the box) and in the
    # density rows the right-hand side is zero up to rounding, where a
    # relative L1 measures noise; bound the error by the largest entry
    y_ref, m_ref = orc.rhs(x0)
    yd = torch.empty(x0.size, dtype=torch.float64, device="cuda:0")
    m = ctx.rhs(dev(x0), yd)
    # (the face and volume terms, each ~n |p|, cancel to the result)
    assert np.abs(yd.cpu().numpy() - y_ref).max() < 1e-10 * np.abs(y_ref).max()
    assert m == pytest.approx(m_ref, rel=1e-12)
    y_ref, m_ref = orc.rhs(x)
    m = ctx.rhs(dev(x), yd)
    assert rel_l1(yd.cpu().numpy(), y_ref) < 1e-12
    assert m == pytest.approx(m_ref, rel=1e-12)
    c32 = Context(case.mesh, case.order, device=0, precision=FP32_BULK)
    cases.configure_context(case, c32)
    y32 = torch.empty(x.size, dtype=torch.float64, device="cuda:0")
    c32.rhs(dev(x), y32)
    assert rel_l1(y32.cpu().numpy(), y_ref) < 1e-5
