"""rkdg_limit_static against rkdg_limit.

rkdg_limit_static serves callers that may not allocate device memory while
they step (their device memory belongs to another allocator, or their loop
must not stall on cudaMalloc/cudaFree): it keeps the cell means in the
library's fixed device array instead of context memory.  Checked here through
the C ABI: bit-identical to rkdg_limit on two calls in a row, and meshes
beyond the fixed capacity are rejected with x untouched."""
import numpy as np
import pytest
import torch

from rkdg3d_gb300 import cases
from rkdg3d_gb300 import mesh as M
from rkdg3d_gb300.solver import (BC_SLIP, FUN_BJ, FUN_MICHALAK, FUN_VENKATAKRISHNAN, IND_BJ,
                                 LIM_FINDIFF, LIM_MULTI, RS_RUSANOV, Context, RkdgError)
from tests.helpers import random_state

pytestmark = pytest.mark.gpu

# RKDG_LIMIT_STATIC_MAX_VALUES and RKDG_ERR_INVALID in include/rkdg_gpu.h
MAX_VALUES = 1 << 21
RKDG_ERR_INVALID = 1


def _state(ctx, case, seed):
    """Sod-like jump plus nodal noise: limits in many cells."""
    X = ctx.node_coords()
    x = random_state(X, seed=seed, amp=0.2, vel=0.3).reshape(ctx.neq, -1)
    jump = np.where(X[0] < 0.5, 1.0, 0.3)
    x = x * jump[None, :]
    return torch.tensor(x.ravel(), dtype=torch.float64, device="cuda:0")


def _case(geom, order, lim, fun):
    bcs = []
    if geom == M.GEOM_CUBE:
        mesh = M.hex_grid(5, 4, 3, periodic=(True, True, True))
    elif geom == M.GEOM_SQUARE:
        mesh = M.quad_grid(24, 5, 0, 1, 0, 0.2, periodic=(True, True))
    else:
        mesh = M.tri_grid(12, 6, 0, 1, 0, 0.5, jitter=0.2)
        bcs = [(a, BC_SLIP, None) for a in (1, 2, 3, 4)]
    return cases.Case("limit_static", mesh, order, RS_RUSANOV, 0, bcs=bcs,
                      limiter=(lim, IND_BJ, fun, 1, 0))


@pytest.mark.parametrize("geom,order,lim,fun", [
    (M.GEOM_SQUARE, 1, LIM_MULTI, FUN_BJ),
    (M.GEOM_SQUARE, 2, LIM_FINDIFF, FUN_MICHALAK),
    (M.GEOM_TRIANGLE, 1, LIM_MULTI, FUN_VENKATAKRISHNAN),
    (M.GEOM_CUBE, 1, LIM_MULTI, FUN_MICHALAK),
])
def test_limit_static_equals_limit(cuda, geom, order, lim, fun):
    case = _case(geom, order, lim, fun)
    ctx = Context(case.mesh, case.order, device=0)
    cases.configure_context(case, ctx)
    changed = 0
    for call, seed in enumerate((11, 12)):
        a = _state(ctx, case, seed)
        b = a.clone()
        x0 = a.clone()
        ctx.limit(a)
        ctx.limit_static(b)
        torch.cuda.synchronize()
        assert torch.equal(a, b), call
        changed += int(not torch.equal(a, x0))
    # the inputs were rough enough for the limiter to act
    assert changed == 2
    # and again on the limited output, straight after
    c = b.clone()
    ctx.limit(b)
    ctx.limit_static(c)
    assert torch.equal(b, c)


def test_limit_static_allocates_nothing(cuda):
    """After one warm call (module load, address look-up), further calls
    leave the device's free memory unchanged: the cell means go to the fixed
    array, nothing is allocated or freed."""
    case = _case(M.GEOM_SQUARE, 1, LIM_MULTI, FUN_BJ)
    ctx = Context(case.mesh, case.order, device=0)
    cases.configure_context(case, ctx)
    x = _state(ctx, case, 13)
    ctx.limit_static(x)
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for _ in range(5):
        ctx.limit_static(x)
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0


def test_limit_static_rejects_oversize_mesh(cuda):
    # 725 x 725 quads, 4 equations: 2,102,500 > 2^21 means
    mesh = M.quad_grid(725, 725, 0, 1, 0, 1, periodic=(True, True))
    assert 4 * mesh.num_elements > MAX_VALUES
    case = cases.Case("oversize", mesh, 1, RS_RUSANOV, 0, limiter=(LIM_MULTI, IND_BJ, FUN_BJ, 1, 0))
    ctx = Context(case.mesh, case.order, device=0)
    cases.configure_context(case, ctx)
    x = torch.ones(ctx.neq * ctx.ndofs, dtype=torch.float64, device="cuda:0")
    with pytest.raises(RkdgError) as ei:
        ctx.limit_static(x)
    assert ei.value.status == RKDG_ERR_INVALID
    assert torch.equal(x, torch.ones_like(x))
