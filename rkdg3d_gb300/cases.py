"""Seeded synthetic case set-ups (meshes, initial states, boundary conditions,
scheme choices) for the benchmark configurations.

No public dataset is involved: every configuration is generated here from its
stated sizes and seeds.  Initial states are projected nodally, which is what
MFEM's ``ProjectCoefficient`` does for a nodal L2 space (case_manager.cpp:
515-516).  Conservative variables are [rho, rho*u, rho*v, (rho*w), E] with
E = p/(gamma-1)*(1 - rho*b) + rho*|u|^2/2 (ComputeEnergy, physics.cpp:128-131).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from . import mesh as M
from .solver import (AVG_EINFELDT, AVG_TRRS, BC_OPEN, BC_SLIP, BC_SUPERSONIC_INLET, FUN_BJ,
                     FUN_MICHALAK, FUN_VENKATAKRISHNAN, IND_BJ, IND_NOWHERE, LIM_FINDIFF,
                     LIM_MULTI, RS_HLL, RS_HLLC, RS_RUSANOV, TABLEAU_SSPRK3)


@dataclass
class Case:
    name: str
    mesh: M.Mesh
    order: int
    rsolver: int
    averaging: int
    gamma: float = 1.4
    covolume: float = 0.0
    bcs: list = field(default_factory=list)      # (attr, type, state or None)
    limiter: tuple = (LIM_FINDIFF, IND_NOWHERE, FUN_MICHALAK, 1, 0)
    tableau: tuple = TABLEAU_SSPRK3
    t_end: float = 0.2
    cfl: float = 0.3
    dt_mode: int = 0          # 0 dynamic, 1 CFL once then fixed, 2 fixed dt0
    dt0: float = 0.0
    max_steps: int = 0
    ic: object = None         # callable(coords[dim, NDofs]) -> primitive (rho, u, v, [w], p)
    solver_quirks: int = 0    # RKDG_QUIRK_* of rkdg_set_solver_quirks
    gas_constant: float = 1.0  # R of the pressure / temperature boundary conditions

    @property
    def dim(self) -> int:
        return self.mesh.dim


def energy(rho, vel, p, gamma, b):
    ke = 0.5 * rho * sum(v * v for v in vel)
    return p / (gamma - 1.0) * (1.0 - rho * b) + ke


def conservative(prim, gamma, b):
    rho, *vel, p = prim
    out = [rho] + [rho * v for v in vel] + [energy(rho, vel, p, gamma, b)]
    return np.concatenate([np.asarray(o, dtype=np.float64).ravel() for o in out])


def project(case: Case, coords: np.ndarray) -> np.ndarray:
    """Nodal projection of the primitive IC; returns the byNODES state."""
    prim = case.ic(coords)
    return conservative(prim, case.gamma, case.covolume)


def supersonic_inlet_state(rho, u, v, w, p, gamma, dim):
    """Boundary state exactly as CaseManager builds it for supersonicInlet
    (case_manager.cpp:743-749): E = p/(gamma-1) + rho*(u^2+v^2)/2."""
    st = [rho, rho * u, rho * v] + ([rho * w] if dim == 3 else [])
    st.append(p / (gamma - 1.0) + 0.5 * rho * (u * u + v * v))
    return np.array(st)


# ---- configurations ------------------------------------------------------------
def sod(nx=200, ny=4, order=1, rsolver=RS_HLLC, averaging=AVG_EINFELDT, function=FUN_BJ,
        tableau=TABLEAU_SSPRK3, t_end=0.2, cfl=0.3) -> Case:
    """2D Sod shock tube, nx x ny quads on [0,1]x[0,0.02]; slip walls top and
    bottom, open ends; Multi limiter with the BJ-family indicator."""
    mesh = M.quad_grid(nx, ny, 0.0, 1.0, 0.0, 0.02)

    def ic(x):
        left = x[0] < 0.5
        rho = np.where(left, 1.0, 0.125)
        p = np.where(left, 1.0, 0.1)
        z = np.zeros_like(rho)
        return rho, z, z, p

    return Case("sod", mesh, order, rsolver, averaging,
                bcs=[(1, BC_SLIP, None), (3, BC_SLIP, None), (2, BC_OPEN, None), (4, BC_OPEN, None)],
                limiter=(LIM_MULTI, IND_BJ, function, 1, 0), tableau=tableau, t_end=t_end, cfl=cfl,
                ic=ic)


def pulse3d(n=64, order=2, steps=500, cfl=0.2) -> Case:
    """3D periodic acoustic pulse on an n^3 hex mesh over [0,1]^3:
    rho = 1 + 0.01*exp(-|x-0.5|^2/0.005), p = rho^gamma, u = 0; Rusanov, no
    limiter, SSP-RK3 with dt fixed from CFL at t = 0."""
    mesh = M.hex_grid(n, n, n)
    gamma = 1.4

    def ic(x):
        r2 = (x[0] - 0.5) ** 2 + (x[1] - 0.5) ** 2 + (x[2] - 0.5) ** 2
        rho = 1.0 + 0.01 * np.exp(-r2 / 0.005)
        z = np.zeros_like(rho)
        return rho, z, z, z, rho ** gamma

    return Case("pulse3d", mesh, order, RS_RUSANOV, AVG_TRRS, gamma=gamma,
                limiter=(LIM_FINDIFF, IND_NOWHERE, FUN_MICHALAK, 1, 0), t_end=1e30, cfl=cfl,
                dt_mode=1, max_steps=steps, ic=ic)


def gaussian_pulses(n=32, order=1, seed=0, steps=200, cfl=0.2, npulse=8) -> Case:
    """3D periodic box [0,1]^3 on an n^3 hex mesh with
    rho = 1 + sum_i a_i exp(-d_i^2 / w_i^2), p = rho^gamma, u = 0, where d_i is
    the periodic (minimum-image) distance to centre c_i; a_i ~ U[0.005, 0.02],
    w_i ~ U[0.03, 0.08], c_i ~ U[0,1]^3, drawn from
    numpy.random.default_rng(seed) in the order a, w, c.  HLLC + TRRS,
    Multi limiter with the Venkatakrishnan indicator function, SSP-RK3 with
    dt fixed from CFL at t = 0, `steps` steps (the adjoint workload)."""
    rng = np.random.default_rng(seed)
    amp = rng.uniform(0.005, 0.02, npulse)
    wid = rng.uniform(0.03, 0.08, npulse)
    cen = rng.uniform(0.0, 1.0, (npulse, 3))
    mesh = M.hex_grid(n, n, n)
    gamma = 1.4

    def ic(x):
        rho = np.ones_like(x[0])
        for a, w, c in zip(amp, wid, cen):
            d2 = np.zeros_like(x[0])
            for k in range(3):
                dk = np.abs(x[k] - c[k])
                dk = np.minimum(dk, 1.0 - dk)
                d2 += dk * dk
            rho += a * np.exp(-d2 / (w * w))
        z = np.zeros_like(rho)
        return rho, z, z, z, rho ** gamma

    return Case(f"gaussian_pulses{seed}", mesh, order, RS_HLLC, AVG_TRRS, gamma=gamma,
                limiter=(LIM_MULTI, IND_BJ, FUN_VENKATAKRISHNAN, 1, 0), tableau=TABLEAU_SSPRK3,
                t_end=1e30, cfl=cfl, dt_mode=1, max_steps=steps, ic=ic)


def gaussian_pulses_perturbed(n=32, order=1, seed=0, perturb_seed=1, scale=0.25, steps=200,
                              cfl=0.2) -> Case:
    """The target of the adjoint workload: the seed-``seed`` pulses of
    gaussian_pulses with a seed-``perturb_seed`` perturbation added,
    rho = rho_seed + scale * (rho_perturb_seed - 1), p = rho^gamma, u = 0."""
    base = gaussian_pulses(n, order, seed, steps, cfl)
    pert = gaussian_pulses(n, order, perturb_seed, steps, cfl)
    gamma = base.gamma
    base_ic, pert_ic = base.ic, pert.ic

    def ic(x):
        rho = base_ic(x)[0] + scale * (pert_ic(x)[0] - 1.0)
        z = np.zeros_like(rho)
        return rho, z, z, z, rho ** gamma

    base.name = f"gaussian_pulses{seed}_perturbed{perturb_seed}"
    base.ic = ic
    return base


def double_mach(nx=1024, ny=256, order=1, jitter=0.2, seed=0, t_end=0.2, cfl=0.25) -> Case:
    """Double Mach reflection on [0,4]x[0,1]: jittered triangulation of an
    nx x ny grid; Mach-10 shock at 60 degrees through (1/6, 0); pre-shock
    (rho 1.4, p 1, u 0), post-shock from Rankine-Hugoniot computed below.
    The reference has no time-dependent boundary, so the boundaries are
    static: bottom x<1/6 and left and the top up to the initial shock
    crossing are post-shock supersonic inlets, bottom x>=1/6 is slip, the rest
    of the top and the right side are outlets."""
    gamma = 1.4
    mach = 10.0
    rho1, p1 = 1.4, 1.0
    c1 = np.sqrt(gamma * p1 / rho1)
    ws = mach * c1
    rho2 = rho1 * (gamma + 1) * mach ** 2 / ((gamma - 1) * mach ** 2 + 2)
    p2 = p1 * (2 * gamma * mach ** 2 - (gamma - 1)) / (gamma + 1)
    u2 = ws * (1.0 - rho1 / rho2)
    nrm = np.array([np.sin(np.pi / 3), -np.cos(np.pi / 3)])
    x0 = 1.0 / 6.0
    mesh = M.tri_grid(nx, ny, 0.0, 4.0, 0.0, 1.0, jitter=jitter, seed=seed)
    # re-tag boundary pieces
    mid = mesh.elem_coords  # noqa: F841
    bv = mesh.bdr_vertices
    ba = mesh.bdr_attr.copy()
    vx = np.zeros(int(mesh.elem_vertices.max()) + 1)
    vx[mesh.elem_vertices.ravel()] = mesh.elem_coords[..., 0].ravel()
    xm = 0.5 * (vx[bv[:, 0]] + vx[bv[:, 1]])
    x_top = x0 + 1.0 / np.tan(np.pi / 3)
    ba[(ba == 1) & (xm >= x0)] = 5          # bottom, reflecting part
    ba[(ba == 3) & (xm >= x_top)] = 6       # top, downstream of the shock
    mesh.bdr_attr = ba.astype(np.int32)
    post = supersonic_inlet_state(rho2, u2 * nrm[0], u2 * nrm[1], 0.0, p2, gamma, 2)

    def ic(x):
        behind = nrm[0] * (x[0] - x0) + nrm[1] * x[1] < 0
        rho = np.where(behind, rho2, rho1)
        u = np.where(behind, u2 * nrm[0], 0.0)
        v = np.where(behind, u2 * nrm[1], 0.0)
        p = np.where(behind, p2, p1)
        return rho, u, v, p

    return Case("double_mach", mesh, order, RS_HLL, AVG_TRRS, gamma=gamma,
                bcs=[(1, BC_SUPERSONIC_INLET, post), (4, BC_SUPERSONIC_INLET, post),
                     (3, BC_SUPERSONIC_INLET, post), (5, BC_SLIP, None), (6, BC_OPEN, None),
                     (2, BC_OPEN, None)],
                limiter=(LIM_MULTI, IND_BJ, FUN_VENKATAKRISHNAN, 1, 0), t_end=t_end, cfl=cfl,
                ic=ic)


@dataclass
class BatchCase:
    """Independent 2D Riemann problems solved together (one context)."""
    cases: list
    mesh: M.Mesh
    offsets: np.ndarray
    gammas: np.ndarray
    covolumes: np.ndarray
    order: int
    t_end: float
    cfl: float

    def project(self, coords: np.ndarray) -> np.ndarray:
        """byNODES state of the union mesh from each problem's own IC."""
        nd = (self.order + 1) ** 2
        parts = []
        for p, c in enumerate(self.cases):
            e0, e1 = self.offsets[p], self.offsets[p + 1]
            parts.append(project(c, coords[:, e0 * nd:e1 * nd]).reshape(4, -1))
        return np.concatenate(parts, axis=1).ravel()


def union_mesh(meshes) -> M.Mesh:
    ev, ec, bv, ba = [], [], [], []
    voff = 0
    for m in meshes:
        ev.append(m.elem_vertices + voff)
        ec.append(m.elem_coords)
        bv.append(m.bdr_vertices + voff)
        ba.append(m.bdr_attr)
        voff += int(max(m.elem_vertices.max(), m.bdr_vertices.max() if m.bdr_vertices.size else 0)) + 1
    return M.Mesh(meshes[0].dim, meshes[0].geom, np.concatenate(ev).astype(np.int32),
                  np.concatenate(ec), np.concatenate(bv).astype(np.int32),
                  np.concatenate(ba).astype(np.int32))


def batched_riemann(nprob=256, nmin=100, nmax=2000, seed=0, order=1, t_end=0.15, cfl=0.3,
                    covolume=0.001, tableau=TABLEAU_SSPRK3) -> BatchCase:
    """Uneven batch of 2D Riemann problems: problem i on an N_i x 4 quad mesh
    over [0,1] x [0, 4/N_i], N_i ~ U{nmin..nmax}; rho, p ~ U[0.1,1] and
    u ~ U[-0.5,0.5] on each side, interface ~ U[0.3,0.7]; the first half
    perfect gas (gamma 1.4), the second half covolume b.  HLLC + Einfeldt,
    Multi limiter with the Michalak indicator, slip walls, open ends.  All
    draws come from numpy.random.default_rng(seed) in the order N, rho_L,
    rho_R, p_L, p_R, u_L, u_R, interface."""
    rng = np.random.default_rng(seed)
    N = rng.integers(nmin, nmax + 1, size=nprob)
    rl, rr, pl, pr = rng.uniform(0.1, 1.0, (4, nprob))
    ul, ur = rng.uniform(-0.5, 0.5, (2, nprob))
    xi = rng.uniform(0.3, 0.7, nprob)
    gam = np.full(nprob, 1.4)
    cov = np.where(np.arange(nprob) < nprob // 2, 0.0, covolume)
    cs = []
    for p in range(nprob):
        mesh = M.quad_grid(int(N[p]), 4, 0.0, 1.0, 0.0, 4.0 / N[p])

        def ic(x, p=p):
            left = x[0] < xi[p]
            z = np.zeros_like(x[0])
            return (np.where(left, rl[p], rr[p]), np.where(left, ul[p], ur[p]), z,
                    np.where(left, pl[p], pr[p]))

        cs.append(Case(f"riemann{p}", mesh, order, RS_HLLC, AVG_EINFELDT, gamma=gam[p],
                       covolume=cov[p],
                       bcs=[(1, BC_SLIP, None), (3, BC_SLIP, None), (2, BC_OPEN, None),
                            (4, BC_OPEN, None)],
                       limiter=(LIM_MULTI, IND_BJ, FUN_MICHALAK, 1, 0), tableau=tableau,
                       t_end=t_end, cfl=cfl, ic=ic, solver_quirks=1))
    offs = np.concatenate([[0], np.cumsum([c.mesh.num_elements for c in cs])]).astype(np.int32)
    return BatchCase(cs, union_mesh([c.mesh for c in cs]), offs, gam, cov, order, t_end, cfl)


def configure_batch(bc: BatchCase, ctx) -> None:
    configure_context(bc.cases[0], ctx)
    ctx.batch_setup(bc.offsets, bc.gammas, bc.covolumes)


def configure_oracle(case: Case, oracle) -> None:
    oracle.set_physics(case.rsolver, case.averaging, case.gamma, case.covolume, case.gas_constant)
    for attr, t, st in case.bcs:
        oracle.set_bc(attr, t, st)
    oracle.set_limiter(*case.limiter)
    oracle.set_tableau(*case.tableau)
    oracle.set_solver_quirks(case.solver_quirks)


def configure_context(case: Case, ctx) -> None:
    from .solver import Physics, RiemannSolver
    rs = RiemannSolver(case.averaging)
    rs.code = case.rsolver
    ctx.set_physics(rs, Physics(case.gamma, case.covolume, case.gas_constant))
    ctx.set_solver_quirks(case.solver_quirks)
    for attr, t, st in case.bcs:
        ctx.set_bc(attr, t, st)
    ctx.set_limiter(*case.limiter)
    ctx.set_tableau(*case.tableau)
