"""Batched uneven solves (many independent Riemann problems in one context,
one CUDA-graph launch) against per-problem oracle runs."""
import numpy as np
import pytest
import torch

from oracle.refcpu import Oracle, OracleError
from rkdg3d_gb300 import cases
from rkdg3d_gb300.solver import FP32_BULK, FP64, Context
from tests.helpers import rel_l1

pytestmark = pytest.mark.gpu


def _batch(nprob=8, nmin=20, nmax=60, t_end=0.05, seed=4):
    return cases.batched_riemann(nprob=nprob, nmin=nmin, nmax=nmax, seed=seed, t_end=t_end)


def _ctx(bc, prec=FP64):
    ctx = Context(bc.mesh, bc.order, device=0, precision=prec)
    cases.configure_batch(bc, ctx)
    return ctx


@pytest.mark.parametrize("use_graph", [True, False])
def test_batch_matches_per_problem_oracle(cuda, use_graph):
    """Each problem of the batch is bit-identical to the same problem run
    alone in its own context, and close to its own oracle run.  Limited
    Riemann problems cross the indicator's hard thresholds (the +-1e-3
    switches of indicator_bj.cpp:49-51) at slightly different times under
    different rounding, so GPU and oracle part by ~1e-10 over the run (dt by ~1e-8);
    the oracle itself does not move under a 1e-15 input perturbation."""
    bc = _batch()
    ctx = _ctx(bc)
    x0 = bc.project(ctx.node_coords())
    xd = torch.tensor(x0, dtype=torch.float64, device="cuda")
    info = ctx.batch_run(xd, bc.t_end, bc.cfl, use_graph=use_graph)
    x = xd.cpu().numpy().reshape(4, -1)
    nd = 4
    nfail = 0
    for p, c in enumerate(bc.cases):
        orc = Oracle(c.mesh, c.order)
        cases.configure_oracle(c, orc)
        xp0 = cases.project(c, orc.node_coords())
        try:
            xr, ir = orc.run(xp0, c.t_end, c.cfl)
        except OracleError:
            # the reference exits on this problem; the batch marks it failed
            assert info["steps"][p] < 0, p
            nfail += 1
            continue
        e0, e1 = bc.offsets[p], bc.offsets[p + 1]
        xb = x[:, e0 * nd:e1 * nd]
        single = Context(c.mesh, c.order, device=0, precision=FP64)
        cases.configure_context(c, single)
        xs = torch.tensor(cases.project(c, single.node_coords()), dtype=torch.float64, device="cuda")
        isg = single.run(xs, c.t_end, c.cfl)
        assert info["steps"][p] == isg["steps"] == ir["steps"], p
        assert info["t"][p] == isg["t"], p
        assert np.array_equal(xb, xs.cpu().numpy().reshape(4, -1)), p
        assert info["t"][p] == pytest.approx(ir["t"], rel=1e-7)
        d_gpu = rel_l1(xb[0], xr[:orc.ndofs])
        assert d_gpu < 1e-8, (p, d_gpu)
    assert nfail < len(bc.cases)


def test_batch_graph_equals_host_loop(cuda):
    bc = _batch(nprob=6, seed=7)
    ctx = _ctx(bc)
    x0 = bc.project(ctx.node_coords())
    a = torch.tensor(x0, dtype=torch.float64, device="cuda")
    b = a.clone()
    ia = ctx.batch_run(a, bc.t_end, bc.cfl, use_graph=True)
    ib = ctx.batch_run(b, bc.t_end, bc.cfl, use_graph=False)
    assert np.array_equal(ia["steps"], ib["steps"])
    assert torch.equal(torch.nan_to_num(a), torch.nan_to_num(b))


def test_batch_mixed_close_to_fp64(cuda):
    bc = _batch(nprob=6, seed=9)
    c64, c32 = _ctx(bc, FP64), _ctx(bc, FP32_BULK)
    x0 = bc.project(c64.node_coords())
    a = torch.tensor(x0, dtype=torch.float64, device="cuda")
    b = a.clone()
    ia = c64.batch_run(a, bc.t_end, bc.cfl)
    ib = c32.batch_run(b, bc.t_end, bc.cfl)
    A = a.cpu().numpy().reshape(4, -1)
    B = b.cpu().numpy().reshape(4, -1)
    for p in range(len(bc.cases)):
        if ia["steps"][p] < 0 or ib["steps"][p] < 0:
            continue
        e0, e1 = bc.offsets[p] * 4, bc.offsets[p + 1] * 4
        assert rel_l1(B[0, e0:e1], A[0, e0:e1]) < 1e-4, p


def test_batch_full_size(cuda):
    """The batched workload at full size: 256 Riemann problems on N_i x 4
    strips, N_i ~ U{100..2000} (about 1.08 M elements), t_end 0.15, FP64, one
    graph launch.  Sampled problems are bit-identical to the same problem run
    alone; the two smallest are checked against the oracle."""
    bc = cases.batched_riemann(nprob=256, nmin=100, nmax=2000, seed=0, t_end=0.15)
    ctx = _ctx(bc)
    x0 = bc.project(ctx.node_coords())
    xd = torch.tensor(x0, dtype=torch.float64, device="cuda")
    info = ctx.batch_run(xd, bc.t_end, bc.cfl, use_graph=True)
    x = xd.cpu().numpy().reshape(4, -1)
    nd = 4
    sizes = np.diff(bc.offsets)
    ok = np.flatnonzero(info["steps"] > 0)
    assert ok.size > 200
    rng = np.random.default_rng(0)
    sample = set(rng.choice(ok, 3, replace=False).tolist())
    sample.add(int(ok[np.argmax(sizes[ok])]))
    smallest = ok[np.argsort(sizes[ok])[:2]].tolist()
    for p in sorted(sample | set(smallest)):
        c = bc.cases[p]
        e0, e1 = bc.offsets[p], bc.offsets[p + 1]
        xb = x[:, e0 * nd:e1 * nd]
        single = Context(c.mesh, c.order, device=0, precision=FP64)
        cases.configure_context(c, single)
        xs = torch.tensor(cases.project(c, single.node_coords()), dtype=torch.float64, device="cuda")
        isg = single.run(xs, c.t_end, c.cfl)
        assert info["steps"][p] == isg["steps"], p
        assert info["t"][p] == isg["t"], p
        assert np.array_equal(xb, xs.cpu().numpy().reshape(4, -1)), p
        if p in smallest:
            orc = Oracle(c.mesh, c.order)
            cases.configure_oracle(c, orc)
            xr, ir = orc.run(cases.project(c, orc.node_coords()), c.t_end, c.cfl)
            assert info["steps"][p] == ir["steps"], p
            assert rel_l1(xb[0], xr[:orc.ndofs]) < 1e-8, p


def test_batch_nonconforming(cuda):
    """A batch whose problems are adapted meshes (a few elements at the
    interface refined, leaving hanging faces): each problem bit-identical to
    the same problem alone, and close to its own oracle run.  Hanging faces
    are paired by position when the mesh is uploaded, so the problems sit in
    disjoint regions (problem p shifted by 2p in y; the initial states depend
    on x only)."""
    from rkdg3d_gb300 import mesh as M
    bc = _batch(nprob=4, nmin=16, nmax=30)
    for p, c in enumerate(bc.cases):
        nx = c.mesh.num_elements // 4
        m = M.refine_nc(c.mesh, [nx // 2 - 1, nx // 2, nx + nx // 2])
        c.mesh = M.Mesh(m.dim, m.geom, m.elem_vertices, m.elem_coords + np.array([0.0, 2.0 * p]),
                        m.bdr_vertices, m.bdr_attr)
    offs = np.concatenate([[0], np.cumsum([c.mesh.num_elements for c in bc.cases])]).astype(np.int32)
    bc = cases.BatchCase(bc.cases, cases.union_mesh([c.mesh for c in bc.cases]), offs, bc.gammas,
                         bc.covolumes, bc.order, bc.t_end, bc.cfl)
    ctx = _ctx(bc)
    xd = torch.tensor(bc.project(ctx.node_coords()), dtype=torch.float64, device="cuda")
    info = ctx.batch_run(xd, bc.t_end, bc.cfl)
    x = xd.cpu().numpy().reshape(4, -1)
    nd, nok = 4, 0
    for p, c in enumerate(bc.cases):
        orc = Oracle(c.mesh, c.order)
        cases.configure_oracle(c, orc)
        try:
            xr, ir = orc.run(cases.project(c, orc.node_coords()), c.t_end, c.cfl)
        except OracleError:
            assert info["steps"][p] < 0, p
            continue
        e0, e1 = bc.offsets[p], bc.offsets[p + 1]
        xb = x[:, e0 * nd:e1 * nd]
        single = Context(c.mesh, c.order, device=0, precision=FP64)
        cases.configure_context(c, single)
        xs = torch.tensor(cases.project(c, single.node_coords()), dtype=torch.float64, device="cuda")
        isg = single.run(xs, c.t_end, c.cfl)
        assert info["steps"][p] == isg["steps"] == ir["steps"], p
        assert np.array_equal(xb, xs.cpu().numpy().reshape(4, -1)), p
        assert rel_l1(xb[0], xr[:orc.ndofs]) < 1e-8, p
        nok += 1
    assert nok >= 2


def test_batch_rejects_problems_joined_by_hanging_faces(cuda):
    """Offsets that put the two sides of a hanging face into different
    problems are refused."""
    from rkdg3d_gb300 import mesh as M
    from rkdg3d_gb300.solver import RkdgError
    c = _batch(nprob=1, nmin=8, nmax=8).cases[0]
    m = M.refine_nc(c.mesh, [31])  # the corner element: its four children are the last elements
    ctx = Context(m, 1, device=0)
    cases.configure_context(c, ctx)
    with pytest.raises(RkdgError, match="hanging face"):
        ctx.batch_setup([0, m.num_elements - 4, m.num_elements], [1.4, 1.4], [0.0, 0.0])
