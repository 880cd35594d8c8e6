"""CPU tests of the oracle (no GPU): known-answer physics checks, MFEM-
semantics restatements and the committed golden vectors."""
import os

import numpy as np
import pytest

from oracle.refcpu import Oracle, OracleError
from rkdg3d_gb300 import cases
from rkdg3d_gb300 import mesh as M
from rkdg3d_gb300.solver import (AVG_EINFELDT, AVG_TRRS, BC_SLIP, FUN_MICHALAK, IND_BJ,
                                 LIM_FINDIFF, LIM_MULTI, IND_NOWHERE, RS_HLL, RS_HLLC, RS_LLF,
                                 RS_RUSANOV, TABLEAU_SSPRK3)
from tests import exact_riemann
from tests.golden.make_golden import golden_cases, initial_state
from tests.helpers import periodic_case, random_state, rel_l1, walled_case

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "golden.npz")


def _oracle(case):
    o = Oracle(case.mesh, case.order)
    cases.configure_oracle(case, o)
    return o


def _flux(u, n, gamma=1.4, b=0.0):
    dim = n.shape[-1]
    rho = u[:, 0]
    m = u[:, 1:1 + dim]
    E = u[:, 1 + dim]
    p = (gamma - 1) * (E - 0.5 * (m * m).sum(1) / rho) / (1 - rho * b)
    mn = (m * n).sum(1)
    out = np.zeros_like(u)
    out[:, 0] = mn
    out[:, 1:1 + dim] = mn[:, None] * m / rho[:, None] + p[:, None] * n
    out[:, 1 + dim] = mn * (E + p) / rho
    return out


@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("rs", [RS_RUSANOV, RS_LLF, RS_HLL, RS_HLLC])
@pytest.mark.parametrize("avg", [AVG_TRRS, AVG_EINFELDT])
def test_riemann_consistency(dim, rs, avg):
    """F(u, u, n) = F(u).n for every solver (face flux consistency)."""
    case = periodic_case(M.GEOM_CUBE if dim == 3 else M.GEOM_SQUARE, 3, 1, rs, avg)
    o = _oracle(case)
    rng = np.random.default_rng(1)
    n = 500
    u = cases.conservative([rng.uniform(0.3, 2, n), *rng.uniform(-1, 1, (dim, n)),
                            rng.uniform(0.2, 2, n)], 1.4, 0.0).reshape(dim + 2, n).T.copy()
    nor = rng.normal(size=(n, dim))
    nor /= np.linalg.norm(nor, axis=1, keepdims=True)
    f, s = o.riemann(u, u.copy(), nor)
    if rs != RS_HLLC:  # HLLC returns max(SL, SR), negative in supersonic reverse flow (Q2)
        assert np.all(s > 0)
    assert np.allclose(f, _flux(u, nor), rtol=1e-11, atol=1e-12)


@pytest.mark.parametrize("rs", [RS_RUSANOV, RS_LLF, RS_HLL, RS_HLLC])
def test_riemann_rotation_invariance_2d(rs):
    """Rotating the frame rotates the momentum flux and leaves the rest."""
    o = _oracle(periodic_case(M.GEOM_SQUARE, 3, 1, rs))
    rng = np.random.default_rng(2)
    n = 300
    mk = lambda: cases.conservative([rng.uniform(0.3, 2, n), *rng.uniform(-1, 1, (2, n)),
                                     rng.uniform(0.2, 2, n)], 1.4, 0.0).reshape(4, n).T.copy()
    u1, u2 = mk(), mk()
    nor = rng.normal(size=(n, 2))
    nor /= np.linalg.norm(nor, axis=1, keepdims=True)
    th = 0.7
    R = np.array([[np.cos(th), -np.sin(th)], [np.sin(th), np.cos(th)]])
    rot = lambda u: np.concatenate([u[:, :1], u[:, 1:3] @ R.T, u[:, 3:]], 1)
    f, _ = o.riemann(u1, u2, nor)
    fr, _ = o.riemann(rot(u1), rot(u2), nor @ R.T)
    assert np.allclose(fr, rot(f), rtol=1e-10, atol=1e-11)


@pytest.mark.parametrize("geom,order", [(M.GEOM_SQUARE, 1), (M.GEOM_SQUARE, 2),
                                        (M.GEOM_TRIANGLE, 1), (M.GEOM_TRIANGLE, 2),
                                        (M.GEOM_CUBE, 1), (M.GEOM_CUBE, 2)])
@pytest.mark.parametrize("rs", [RS_RUSANOV, RS_HLLC])
def test_free_stream_rest_state(geom, order, rs):
    """A uniform state at rest in a slip-walled box has a zero right-hand side."""
    case = walled_case(geom, 3, order, rs, bc=BC_SLIP)
    o = _oracle(case)
    X = o.node_coords()
    one = np.ones(X.shape[1])
    x = cases.conservative([1.3 * one] + [0 * one] * case.dim + [0.8 * one], 1.4, 0.0)
    y, _ = o.rhs(x)
    assert np.abs(y).max() < 1e-11


@pytest.mark.parametrize("geom,order", [(M.GEOM_SQUARE, 1), (M.GEOM_SQUARE, 3), (M.GEOM_CUBE, 2)])
def test_free_stream_periodic_uniform_flow(geom, order):
    case = periodic_case(geom, 3, order, RS_HLLC)
    o = _oracle(case)
    X = o.node_coords()
    one = np.ones(X.shape[1])
    x = cases.conservative([one] + [0.3 * one] * case.dim + [one], 1.4, 0.0)
    y, _ = o.rhs(x)
    assert np.abs(y).max() < 1e-11


@pytest.mark.parametrize("geom,order", [(M.GEOM_SQUARE, 2), (M.GEOM_CUBE, 1)])
def test_discrete_conservation(geom, order):
    """sum_e sum_j (int phi_j) dU_j/dt = 0 on a periodic mesh."""
    case = periodic_case(geom, 4, order, RS_HLL)
    o = _oracle(case)
    x = random_state(o.node_coords(), seed=5, amp=0.1, vel=0.2)
    y, _ = o.rhs(x)
    d = o.totals(y)
    assert np.abs(d).max() < 1e-13 * np.abs(o.totals(x)).max() * 1e2


def test_gl_nodes_and_triangle_nodes():
    """Node positions of DG_FECollection's Gauss-Legendre bases."""
    m = M.quad_grid(1, 1)
    o = Oracle(m, 1)
    X = o.node_coords()
    g = 0.5 * (1 - 1 / np.sqrt(3))
    assert np.allclose(sorted(set(np.round(X[0], 14))), [g, 1 - g])
    t = M.tri_grid(1, 1)
    o = Oracle(t, 1)
    X = o.node_coords()[:, :3]   # first triangle (0,0),(1,0),(1,1): x = xi + eta, y = eta
    op = np.array([g, 1 - g])
    w = 2 * op[0] + op[1]
    ref = np.array([[op[0] / w, op[0] / w], [op[1] / w, op[0] / w], [op[0] / w, op[1] / w]])
    phys = np.stack([ref[:, 0] + ref[:, 1], ref[:, 1]], 0)
    assert np.allclose(X, phys, atol=1e-14)


def test_sod_against_exact_solution():
    """Q1 Sod (200 x 4, HLLC, limited) density is close to the exact solution."""
    case = cases.sod(nx=200, ny=4, rsolver=RS_HLLC, averaging=AVG_TRRS, function=FUN_MICHALAK,
                     tableau=TABLEAU_SSPRK3, t_end=0.2)
    o = _oracle(case)
    X = o.node_coords()
    x0 = cases.project(case, X)
    x, info = o.run(x0, case.t_end, case.cfl)
    t = info["sum_dt"]
    rho = x[:o.ndofs]
    ex = exact_riemann.sample(X[0], t, 0.5, (1.0, 0.0, 1.0), (0.125, 0.0, 0.1))[0]
    l1 = np.mean(np.abs(rho - ex))
    assert l1 < 0.01, l1
    assert np.all(rho > 0.1) and np.all(rho < 1.05)


def test_sod_totals_conserved():
    case = cases.sod(nx=50, ny=2, t_end=0.05)
    o = _oracle(case)
    x0 = cases.project(case, o.node_coords())
    t0 = o.totals(x0)
    x, _ = o.run(x0, case.t_end, case.cfl)
    t1 = o.totals(x)
    # mass and energy fluxes through the open ends are zero before the waves arrive
    assert abs(t1[0] - t0[0]) < 1e-14 and abs(t1[3] - t0[3]) < 1e-14


def test_limiter_nowhere_findiff_is_identity():
    case = cases.sod(nx=20, ny=2)
    case.limiter = (LIM_FINDIFF, IND_NOWHERE, FUN_MICHALAK, 1, 0)
    o = _oracle(case)
    x = random_state(o.node_coords(), seed=2)
    assert np.array_equal(o.limit(x), x)


def test_limiter_keeps_means():
    case = cases.sod(nx=30, ny=2)
    case.limiter = (LIM_MULTI, IND_BJ, FUN_MICHALAK, 1, 0)
    o = _oracle(case)
    x = random_state(o.node_coords(), seed=4)
    m0 = o.means(x)
    m1 = o.means(o.limit(x))
    assert np.allclose(m0, m1, rtol=1e-13, atol=1e-14)


@pytest.mark.parametrize("name", list(golden_cases()))
def test_golden_vectors(name):
    g = np.load(GOLDEN)
    case, seed, dt = golden_cases()[name]
    o = _oracle(case)
    x = initial_state(case, o, seed)
    assert np.array_equal(x, g[f"{name}/x"])
    y, mcs = o.rhs(x)
    assert rel_l1(y, g[f"{name}/rhs"]) < 1e-14
    assert mcs == pytest.approx(g[f"{name}/mcs"][0], rel=1e-15)
    assert rel_l1(o.limit(x), g[f"{name}/limited"]) < 1e-14
    xs, _ = o.step(x, dt)
    assert rel_l1(xs, g[f"{name}/step"]) < 1e-14


def _bc_oracle(dim, bctype, params, gamma=1.4, R=1.0):
    geom, n = (M.GEOM_CUBE, 3) if dim == 3 else (M.GEOM_SQUARE, 3)
    case = walled_case(geom, n, 1, 0)
    orc = Oracle(case.mesh, case.order)
    orc.set_physics(0, 0, gamma, 0.0, R)
    orc.set_bc(1, bctype, params)
    return orc


def _prim(s, gamma, dim):
    rho = s[0]
    u = s[1:1 + dim] / rho
    p = (gamma - 1) * (s[-1] - 0.5 * rho * u @ u)
    return rho, u, p


@pytest.mark.parametrize("dim", [2, 3])
def test_bc_subsonic_inlets_known_answers(dim):
    """subsonicInlet{Total,Fixed}Pressure: the ghost state keeps the velocity,
    sits at T = TTot / (1 + (g-1)/2 M^2) with M^2 = MT^2 / (1 - (g-1)/2 MT^2),
    MT^2 = |u|^2 / (g R TTot), and has p = pFix, or p = pTot (T/TTot)^(g/(g-1))."""
    g, R = 1.4, 0.7
    s1 = cases.conservative([np.array([1.1]), *[np.array([v]) for v in (0.2, -0.1, 0.15)[:dim]],
                             np.array([0.9])], g, 0.0).ravel()
    nor = np.zeros(dim)
    nor[0] = -1.0
    for bctype, pv, TTot in ((6, 1.3, 1.2), (7, 0.8, 1.2)):
        s2 = _bc_oracle(dim, bctype, [pv, TTot], g, R).right_state(1, s1, nor)
        rho2, u2, p2 = _prim(s2, g, dim)
        u1 = s1[1:1 + dim] / s1[0]
        assert np.allclose(u2, u1, rtol=1e-14, atol=0)
        mt2 = u1 @ u1 / (g * R * TTot)
        m2 = mt2 / (1 - 0.5 * (g - 1) * mt2)
        T = TTot / (1 + 0.5 * (g - 1) * m2)
        assert p2 / (rho2 * R) == pytest.approx(T, rel=1e-13)
        want = pv * (T / TTot) ** (g / (g - 1)) if bctype == 6 else pv
        assert p2 == pytest.approx(want, rel=1e-13)


@pytest.mark.parametrize("dim", [2, 3])
def test_bc_outlets_known_answers(dim):
    """fixedPressureOutlet: ghost pressure pFix at the interior velocity.
    totalPressureFixedTemperatureOutlet, subsonic: p + rho |u|^2 / 2 = pTot at
    the interior velocity.  subsonicInlet: own + ghost = 2 * fixed in the
    rotated frame (for a normal along x: componentwise)."""
    g = 1.4
    s1 = cases.conservative([np.array([0.9]), *[np.array([v]) for v in (0.3, 0.1, -0.2)[:dim]],
                             np.array([1.1])], g, 0.0).ravel()
    nor = np.zeros(dim)
    nor[0] = 1.0
    u1 = s1[1:1 + dim] / s1[0]
    s2 = _bc_oracle(dim, 8, [0.7]).right_state(1, s1, nor)
    rho2, u2, p2 = _prim(s2, g, dim)
    assert p2 == pytest.approx(0.7, rel=1e-13)
    assert np.allclose(u2, u1, rtol=1e-14, atol=0)
    s2 = _bc_oracle(dim, 9, [1.3, 1.0]).right_state(1, s1, nor)
    rho2, u2, p2 = _prim(s2, g, dim)
    assert np.allclose(u2, u1, rtol=1e-14, atol=0)
    assert p2 + 0.5 * rho2 * u2 @ u2 == pytest.approx(1.3, rel=1e-13)
    fixed = np.array([1.0, 0.2, 0.05, 0.0, 2.6])[[0, *range(1, 1 + dim), 4]]
    s2 = _bc_oracle(dim, 5, fixed).right_state(1, s1, nor)
    assert np.allclose(s1 + s2, 2 * fixed, rtol=1e-14, atol=1e-15)


def test_linearize_keeps_means_and_is_linear():
    """Multi + linearize on Q1 quads (Nowhere indicator: multiplier 1): the
    means stay, and every variable becomes linear in the reference
    coordinates (the bilinear coefficient vanishes)."""
    case = periodic_case(M.GEOM_SQUARE, 4, 1, 0)
    orc = Oracle(case.mesh, case.order)
    cases.configure_oracle(case, orc)
    orc.set_limiter(1, 0, 2, 0, 2)
    x = random_state(orc.node_coords(), seed=2)
    y = orc.limit(x)
    assert np.allclose(orc.means(y), orc.means(x), rtol=0, atol=1e-14)
    v = y.reshape(orc.neq, -1, 4)  # nodes (x0,y0), (x1,y0), (x0,y1), (x1,y1)
    assert np.allclose(v[..., 0] - v[..., 1] - v[..., 2] + v[..., 3], 0.0, atol=1e-13)
    orc.set_limiter(1, 0, 2, 0, 0)
    assert not np.allclose(orc.limit(x), y)


@pytest.mark.parametrize("geom,order", [(M.GEOM_SQUARE, 1), (M.GEOM_SQUARE, 2),
                                        (M.GEOM_TRIANGLE, 1), (M.GEOM_TRIANGLE, 2),
                                        (M.GEOM_CUBE, 1)])
def test_shu_indicator_known_answers(geom, order):
    """Shu indicator + FinDiff: a globally linear state extrapolates exactly
    (every stencil difference vanishes) and is left alone; a jump makes the
    cells beside it fall back to their means while the means stay."""
    case = walled_case(geom, 4, order, 0, bc=BC_SLIP)
    orc = Oracle(case.mesh, case.order)
    cases.configure_oracle(case, orc)
    orc.set_limiter(0, 3, 2, 1, 0)
    X = orc.node_coords()
    lin = cases.conservative([1.0 + 0.1 * X[0] + 0.05 * X[1], *[0.02 * X[0] for _ in range(X.shape[0])],
                              1.0 + 0.03 * X[1]], 1.4, 0.0)
    assert np.allclose(orc.limit(lin), lin, rtol=0, atol=1e-14)
    jump = cases.conservative([np.where(X[0] < 0.4, 1.0, 0.2), *[0 * X[0] for _ in range(X.shape[0])],
                               np.where(X[0] < 0.4, 1.0, 0.1)], 1.4, 0.0)
    y = orc.limit(jump)
    assert not np.allclose(y, jump)
    assert np.allclose(orc.means(y), orc.means(jump), rtol=0, atol=1e-13)


# ---- nonconforming (AMR) meshes -------------------------------------------

def _nc_meshes():
    return [(M.hex_grid(3, 3, 3, periodic=(False,) * 3), [13, 4, 22]),
            (M.quad_grid(4, 4), [5, 6, 0]),
            (M.tri_grid(4, 4, 0, 1, 0, 1, jitter=0.2, seed=3), [9, 10, 0])]


def _linear_state(X, dim):
    """Constant velocity, linear density and pressure: every flux component is
    linear in space, so each element's right-hand side depends on that
    element alone and every face rule integrates it exactly."""
    n = X.shape[1]
    rho = 1.0 + 0.1 * X[0] + 0.05 * X[1]
    vel = [np.full(n, 0.3), np.full(n, -0.2)] + ([np.full(n, 0.1)] if dim == 3 else [])
    p = 1.0 + 0.1 * X[1] - 0.07 * X[0] + (0.05 * X[2] if dim == 3 else 0.0)
    return cases.conservative([rho, *vel, p], 1.4, 0.0)


def _open_case(mesh, order):
    from rkdg3d_gb300.solver import BC_OPEN
    attrs = sorted(set(mesh.bdr_attr.tolist()))
    return cases.Case("nc", mesh, order, RS_HLLC, 0, bcs=[(a, BC_OPEN, None) for a in attrs])


@pytest.mark.parametrize("k", [0, 1, 2])
@pytest.mark.parametrize("order", [1, 2])
def test_nc_faces_match_conforming_meshes(k, order):
    """Hanging faces (slave faces integrated from the fine side, the coarse
    element evaluated at the mapped points, master faces skipped): for a
    state whose fluxes are linear, an unrefined element's right-hand side on
    the nonconforming mesh equals the coarse mesh's, and a child's equals the
    fully refined mesh's."""
    base, ref = _nc_meshes()[k]
    nc = M.refine_nc(base, ref)
    full = M.refine_nc(base, range(base.num_elements))
    dim, neq = base.dim, base.dim + 2
    nd = (order + 1) * (order + 2) // 2 if base.geom == M.GEOM_TRIANGLE else (order + 1) ** dim

    def rhs(m):
        o = _oracle(_open_case(m, order))
        y, _ = o.rhs(_linear_state(o.node_coords(), dim))
        return y.reshape(neq, m.num_elements, nd)

    Yb, Yn, Yf = rhs(base), rhs(nc), rhs(full)
    cf = full.elem_coords.mean(1)
    refined = set(ref)
    err = 0.0
    for e in range(nc.num_elements):
        if e < base.num_elements and e not in refined:
            err = max(err, np.abs(Yn[:, e] - Yb[:, e]).max())
        else:
            j = int(np.argmin(np.abs(cf - nc.elem_coords[e].mean(0)).sum(1)))
            err = max(err, np.abs(Yn[:, e] - Yf[:, j]).max())
    assert err < 1e-11 * np.abs(Yb).max()


@pytest.mark.parametrize("geom", [M.GEOM_CUBE, M.GEOM_SQUARE])
def test_nc_free_stream_and_conservation(geom):
    if geom == M.GEOM_CUBE:
        m = M.refine_nc(M.hex_grid(4, 4, 4), [21, 22, 42])
    else:
        m = M.refine_nc(M.quad_grid(5, 5, periodic=(True, True)), [6, 7, 12, 18])
    o = _oracle(cases.Case("nc", m, 2, RS_HLLC, 0))
    X = o.node_coords()
    one = np.ones(X.shape[1])
    y, _ = o.rhs(cases.conservative([1.2 * one] + [0.3 * one] * m.dim + [one], 1.4, 0.0))
    assert np.abs(y).max() < 1e-11
    x = random_state(X, seed=4, amp=0.05, vel=0.1)
    y, _ = o.rhs(x)
    assert np.abs(o.totals(y)).max() < 1e-11 * np.abs(o.totals(x)).max()


def test_nc_mesh_with_uncovered_face_is_rejected():
    """A lone face that is neither inside another element's face nor covered
    by slaves (a gap in the mesh) is an invalid mesh."""
    m = M.hex_grid(3, 3, 3, periodic=(False,) * 3)
    keep = [e for e in range(m.num_elements) if e != 13]  # a hole in the middle
    holed = M.Mesh(3, M.GEOM_CUBE, m.elem_vertices[keep], m.elem_coords[keep], m.bdr_vertices, m.bdr_attr)
    with pytest.raises(Exception):
        Oracle(holed, 1)


# ---- non-parallelogram (bilinear) quadrilaterals --------------------------------

@pytest.mark.parametrize("order", [1, 2, 3])
def test_bilinear_quads_free_stream_and_conservation(order):
    """General quadrilaterals (interior vertices moved): a uniform flow stays
    uniform on a periodic mesh (the collocated metric terms of a bilinear map
    are exact), and the discrete totals are conserved."""
    m = M.perturb(M.quad_grid(6, 6, periodic=(True, True)), 0.03, seed=2)
    X = m.elem_coords
    assert (np.abs(X[:, 0] + X[:, 2] - X[:, 1] - X[:, 3]).max(1) > 1e-6).sum() > 10
    o = _oracle(cases.Case("q", m, order, RS_HLLC, 0))
    Xn = o.node_coords()
    one = np.ones(Xn.shape[1])
    y, _ = o.rhs(cases.conservative([1.1 * one, 0.3 * one, -0.2 * one, one], 1.4, 0.0))
    assert np.abs(y).max() < 1e-11
    x = random_state(Xn, seed=6, amp=0.05, vel=0.1)
    y, _ = o.rhs(x)
    assert np.abs(o.totals(y)).max() < 1e-12 * np.abs(o.totals(x)).max()


@pytest.mark.parametrize("dt_mode", [0, 1, 2])
def test_run_in_pieces_equals_one_run(dt_mode):
    """ref_run_continue with the t and dt a piece returned steps exactly as one
    ref_run (the restart path of main.cpp:461-490 without the frame's limit)."""
    from rkdg3d_gb300 import cases
    case = cases.sod(nx=30, ny=2, t_end=0.05)
    o = Oracle(case.mesh, case.order)
    cases.configure_oracle(case, o)
    x0 = cases.project(case, o.node_coords())
    dt0 = 1e-3 if dt_mode == 2 else 0.0
    x_all, i_all = o.run(x0, case.t_end, case.cfl, dt0=dt0, dt_mode=dt_mode)
    x1, i1 = o.run(x0, case.t_end, case.cfl, dt0=dt0, dt_mode=dt_mode, max_steps=7)
    x2, i2 = o.run_continue(x1, i1["t"], i1["dt"], case.t_end, case.cfl, dt_mode=dt_mode)
    assert i1["steps"] + i2["steps"] == i_all["steps"]
    assert np.array_equal(x2, x_all)
    assert i2["t"] == i_all["t"] and i2["dt"] == i_all["dt"]
    with pytest.raises(OracleError):
        o.run_continue(x1, 0.0, 0.0, case.t_end, case.cfl)
