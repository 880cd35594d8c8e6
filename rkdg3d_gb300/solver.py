"""Host-side mirror of the reference's fe_evolution / riemannsolvers /
averager / limiter / ode_solver interfaces over the GB300 C ABI.

Names, argument meaning and error behaviour follow the reference:

* ``RiemannSolverRusanov/LLF/HLL/HLLC``       (src/riemannsolvers/, factory
  case_manager.cpp:523-543)
* ``FE_Evolution.Mult(x, y)``                  (fe_evolution.hpp:75)
* ``Averager.computeMeanValues`` / ``readElementAverageByNumber``
  (averager.hpp:139-145)
* ``IndicatorNowhere/Everywhere/BJ`` and ``LimiterFinDiff/LimiterMultiplier``
  with ``Limiter.update(x)`` (limiter.hpp:111, factory case_manager.cpp:545-612)
* ``ExplicitRKLimitedSolver(s, a, b, c, limiter)`` with ``Init`` / ``Step``
  (rk_explicit_limited.hpp:46-56)

State vectors are CUDA tensors (float64, contiguous, byNODES layout) or raw
device pointers.  A non-physical state raises :class:`UnphysicalStateError`
where the reference prints the element numbers and calls ``exit(1)``
(face_integrator.cpp:214-218).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _capi
from .mesh import Mesh

RKDG_OK = 0
RKDG_ERR_UNPHYSICAL = 2

RS_RUSANOV, RS_LLF, RS_HLL, RS_HLLC = 0, 1, 2, 3
AVG_TRRS, AVG_EINFELDT = 0, 1
BC_SLIP, BC_OPEN, BC_FIXED_ROTATED, BC_SUPERSONIC_INLET, BC_WALL = 0, 1, 2, 3, 4
# parameters in state: {pTot, TTot}, {pFix, TTot}, {pFix}, {pTot, TFix}
(BC_SUBSONIC_INLET, BC_SUBSONIC_INLET_TOTAL_PRESSURE, BC_SUBSONIC_INLET_FIXED_PRESSURE,
 BC_FIXED_PRESSURE_OUTLET, BC_TOTAL_PRESSURE_OUTLET) = 5, 6, 7, 8, 9
# characteristic outlet, state = the outer conservative state (the ghost state
# enters its computation as the interior state, where the reference reads the
# previous boundary point's)
BC_CHAR_OUTLET = 10
LIM_FINDIFF, LIM_MULTI = 0, 1
IND_NOWHERE, IND_EVERYWHERE, IND_BJ, IND_SHU = 0, 1, 2, 3
FUN_BJ, FUN_VENKATAKRISHNAN, FUN_MICHALAK = 0, 1, 2
QUIRK_MULTIPLIER_ONCE = 1
FP64, FP32_BULK = 0, 1
# flags of set_solver_quirks
QUIRK_HLLC_NEGATIVE_SPEED_OK, QUIRK_NO_INITIAL_LIMIT = 1, 2
TUNE_HEX_KERNEL, TUNE_GENERIC_BLOCK, TUNE_LIMITER_BLOCK = 1, 2, 3
# flags of set_limiter(quirks=...)
QUIRK_MULTIPLIER_ONCE, LIMITER_LINEARIZE = 1, 2

# Butcher tableaux in MFEM lower-triangular packing.
# True SSP-RK3 (Shu-Osher third order) in Butcher form.
TABLEAU_SSPRK3 = (3, [1.0, 0.25, 0.25], [1.0 / 6.0, 1.0 / 6.0, 2.0 / 3.0], [1.0, 0.5])
# The arrays the reference builds for time.order = 3 (case_manager.cpp:871-884),
# read with MFEM's packing by ExplicitRKLimitedSolver::Step (a21=0, a31=1, a32=0).
TABLEAU_REFERENCE_RK3 = (3, [0.0, 1.0, 0.0], [0.1666666666666666, 0.1666666666666666,
                                              0.6666666666666666], [0.0, 0.5])
# time.order = 2 (case_manager.cpp:829-840): a21 = 0.
TABLEAU_REFERENCE_RK2 = (2, [0.0], [0.5, 0.5], [0.0])


class RkdgError(RuntimeError):
    def __init__(self, status: int, message: str, where: int = -1):
        super().__init__(f"rkdg status {status}: {message}")
        self.status = status
        self.where = where


class UnphysicalStateError(RkdgError):
    pass


def _ptr(t) -> int:
    if isinstance(t, int):
        return t
    if hasattr(t, "data_ptr"):
        if not t.is_cuda or not t.is_contiguous():
            raise ValueError("state must be a contiguous CUDA tensor")
        return int(t.data_ptr())
    raise TypeError("expected a CUDA tensor or a device pointer")


class RiemannSolver:
    code = RS_RUSANOV

    def __init__(self, averaging: int = AVG_TRRS):
        self.averaging = averaging


class RiemannSolverRusanov(RiemannSolver):
    code = RS_RUSANOV


class RiemannSolverLLF(RiemannSolver):
    code = RS_LLF


class RiemannSolverHLL(RiemannSolver):
    code = RS_HLL


class RiemannSolverHLLC(RiemannSolver):
    code = RS_HLLC


@dataclass
class Physics:
    gamma: float = 1.4
    covolume: float = 0.0
    gas_constant: float = 1.0


class Context:
    """One device context: mesh tables, physics, boundary conditions, limiter,
    tableau and precision.  Wraps ``rkdg_ctx``."""

    def __init__(self, mesh: Mesh, order: int, device: int = 0, precision: int = FP64):
        L = _capi.load()
        self._L = L
        h = C.c_void_p()
        st = L.rkdg_create(C.byref(h), device)
        if st != RKDG_OK:
            raise RkdgError(st, "rkdg_create failed (no CUDA device?)")
        self.h = h
        self.mesh = mesh.contiguous()
        self.order = order
        self._upload()
        self.set_precision(precision)
        ndofs = C.c_longlong()
        nd = C.c_int()
        neq = C.c_int()
        self._chk(L.rkdg_sizes(self.h, C.byref(ndofs), C.byref(nd), C.byref(neq)))
        self.ndofs, self.nd, self.neq = ndofs.value, nd.value, neq.value
        self.ne = self.mesh.num_elements
        self.dim = self.mesh.dim

    def _upload(self):
        m = self.mesh
        d = _capi.MeshDesc()
        d.dim, d.geom, d.order, d.num_elements = m.dim, m.geom, self.order, m.num_elements
        d.elem_vertices = m.elem_vertices.ctypes.data_as(_capi._ip)
        d.elem_coords = m.elem_coords.ctypes.data_as(_capi._dp)
        d.num_bdr = m.bdr_vertices.shape[0]
        d.bdr_vertices = m.bdr_vertices.ctypes.data_as(_capi._ip)
        d.bdr_attr = m.bdr_attr.ctypes.data_as(_capi._ip)
        self._chk(self._L.rkdg_upload_mesh(self.h, C.byref(d)))

    def update_mesh(self, mesh: Mesh):
        """After an adapt (UpdateAndRebalance, amr.cpp:3-133): rebuild every
        device table for the new (possibly nonconforming) mesh, as
        UpdateAfluxPointer / UpdateInverseMassMatrix do (main.cpp:610-611).
        Physics, boundary conditions, limiter and tableau are kept."""
        self.mesh = mesh.contiguous()
        self._upload()
        ndofs = C.c_longlong()
        self._chk(self._L.rkdg_sizes(self.h, C.byref(ndofs), None, None))
        self.ndofs = ndofs.value
        self.ne = self.mesh.num_elements

    def __del__(self):
        if getattr(self, "h", None) is not None and self.h.value:
            self._L.rkdg_destroy(self.h)
            self.h = None

    def _chk(self, st: int):
        if st != RKDG_OK:
            where = C.c_longlong(-1)
            msg = self._L.rkdg_last_error(self.h, C.byref(where)).decode()
            cls = UnphysicalStateError if st == RKDG_ERR_UNPHYSICAL else RkdgError
            raise cls(st, msg, where.value)

    # -- configuration ------------------------------------------------------
    def set_physics(self, rsolver: RiemannSolver, physics: Physics = Physics()):
        self._chk(self._L.rkdg_set_physics(self.h, rsolver.code, rsolver.averaging, physics.gamma,
                                           physics.covolume, physics.gas_constant))

    def set_bc(self, attr: int, bctype: int, state=None):
        """state: conservative variables, or the boundary condition's
        parameters in its first entries (padded to five values)."""
        arr = None
        if state is not None:
            arr = np.zeros(5, dtype=np.float64)
            v = np.asarray(state, dtype=np.float64).ravel()
            arr[:v.size] = v
        self._chk(self._L.rkdg_set_bc(self.h, attr, bctype,
                                      arr.ctypes.data_as(_capi._dp) if arr is not None else None))
        self._keep_bc = arr

    def set_limiter(self, limiter=LIM_FINDIFF, indicator=IND_NOWHERE, function=FUN_MICHALAK,
                    last_hope=1, quirks=0):
        self._chk(self._L.rkdg_set_limiter(self.h, limiter, indicator, function, last_hope, quirks))

    def set_tableau(self, s, a, b, c):
        a = np.ascontiguousarray(a if len(a) else [0.0], dtype=np.float64)
        b = np.ascontiguousarray(b, dtype=np.float64)
        c = np.ascontiguousarray(c if len(c) else [0.0], dtype=np.float64)
        self._chk(self._L.rkdg_set_tableau(self.h, s, a.ctypes.data_as(_capi._dp),
                                           b.ctypes.data_as(_capi._dp), c.ctypes.data_as(_capi._dp)))

    def set_precision(self, precision: int):
        self._chk(self._L.rkdg_set_precision(self.h, precision))
        self.precision = precision

    def set_solver_quirks(self, flags: int):
        self._chk(self._L.rkdg_set_solver_quirks(self.h, flags))
        self._solver_quirks = int(flags)

    def _initial_limit(self, on: bool):
        q = getattr(self, "_solver_quirks", 0)
        q = (q & ~QUIRK_NO_INITIAL_LIMIT) | (0 if on else QUIRK_NO_INITIAL_LIMIT)
        if q != getattr(self, "_solver_quirks", 0):
            self.set_solver_quirks(q)

    def set_tuning(self, key: int, value: int):
        self._chk(self._L.rkdg_set_tuning(self.h, key, value))

    def autotune(self, x) -> dict:
        """Time the candidate launch shapes on state x and keep the fastest
        (rkdg_autotune); returns the chosen tuning values."""
        hk, gb, lb = C.c_int(), C.c_int(), C.c_int()
        self._chk(self._L.rkdg_autotune(self.h, _ptr(x), C.byref(hk), C.byref(gb), C.byref(lb)))
        return {"hex_kernel": hk.value, "generic_block": gb.value, "limiter_block": lb.value}

    def set_stream(self, stream_ptr: int | None):
        self._chk(self._L.rkdg_set_stream(self.h, stream_ptr))

    # -- queries --------------------------------------------------------------
    @property
    def n(self) -> int:
        return self.ndofs * self.neq

    def node_coords(self) -> np.ndarray:
        out = np.zeros(self.dim * self.ndofs)
        self._chk(self._L.rkdg_node_coords_host(self.h, out.ctypes.data_as(_capi._dp)))
        return out.reshape(self.dim, self.ndofs)

    def hmin(self) -> float:
        v = C.c_double()
        self._chk(self._L.rkdg_hmin(self.h, C.byref(v)))
        return v.value

    def launches(self) -> int:
        return int(self._L.rkdg_kernel_launches(self.h))

    # -- hot path -------------------------------------------------------------
    def rhs(self, x, y) -> float:
        m = C.c_double()
        self._chk(self._L.rkdg_rhs(self.h, _ptr(x), _ptr(y), C.byref(m)))
        return m.value

    def face_speed(self, x) -> float:
        m = C.c_double()
        self._chk(self._L.rkdg_face_speed(self.h, _ptr(x), C.byref(m)))
        return m.value

    def limit(self, x):
        self._chk(self._L.rkdg_limit(self.h, _ptr(x)))

    def limit_static(self, x):
        """Same as limit(), with the cell means in the library's fixed device
        array instead of context memory (no allocation; one call at a time
        per device)."""
        self._chk(self._L.rkdg_limit_static(self.h, _ptr(x)))

    def cell_means(self, x, means):
        self._chk(self._L.rkdg_cell_means(self.h, _ptr(x), _ptr(means)))

    def step(self, x, dt: float) -> float:
        m = C.c_double()
        self._chk(self._L.rkdg_step(self.h, _ptr(x), dt, C.byref(m)))
        return m.value

    def run(self, x, t_end: float, cfl: float = 0.3, dt0: float = 0.0, dt_mode: int = 0,
            max_steps: int = 0, limit_initial: bool = True) -> dict:
        """The reference's time loop (rkdg_run).  limit_initial: limit x once
        before the first dt, as the reference does with the projected initial
        state (main.cpp:264-265); False continues from a state as given."""
        if max_steps <= 0 and not (t_end < 1e20):
            raise ValueError("run() needs a finite t_end or max_steps > 0")
        self._initial_limit(limit_initial)
        steps = C.c_int()
        t = C.c_double()
        dt = C.c_double()
        sdt = C.c_double()
        self._chk(self._L.rkdg_run(self.h, _ptr(x), t_end, cfl, dt0, dt_mode, max_steps,
                                   C.byref(steps), C.byref(t), C.byref(dt), C.byref(sdt)))
        return {"steps": steps.value, "t": t.value, "dt": dt.value, "sum_dt": sdt.value}

    def run_continue(self, x, t0: float, dt: float, t_end: float, cfl: float = 0.3,
                     dt_mode: int = 0, max_steps: int = 0) -> dict:
        """The time loop continued at time t0 with the next dt known
        (rkdg_run_continue): a restart frame's t and dt, or the t and dt that
        the previous piece of a run returned."""
        if max_steps <= 0 and not (t_end < 1e20):
            raise ValueError("run_continue() needs a finite t_end or max_steps > 0")
        steps = C.c_int()
        t = C.c_double()
        dto = C.c_double()
        sdt = C.c_double()
        self._chk(self._L.rkdg_run_continue(self.h, _ptr(x), t0, dt, t_end, cfl, dt_mode, max_steps,
                                            C.byref(steps), C.byref(t), C.byref(dto), C.byref(sdt)))
        return {"steps": steps.value, "t": t.value, "dt": dto.value, "sum_dt": sdt.value}

    def totals(self, x) -> np.ndarray:
        out = np.zeros(self.neq)
        self._chk(self._L.rkdg_totals(self.h, _ptr(x), out.ctypes.data_as(_capi._dp)))
        return out

    def riemann_batch(self, u1, u2, nor, flux, speed):
        n = int(u1.shape[0])
        self._chk(self._L.rkdg_riemann_batch(self.h, n, _ptr(u1), _ptr(u2), _ptr(nor), _ptr(flux),
                                             _ptr(speed)))

    def synchronize(self):
        self._chk(self._L.rkdg_synchronize(self.h))

    # -- discrete adjoint (FP64) ----------------------------------------------
    def rhs_vjp(self, x, kbar, xbar):
        self._chk(self._L.rkdg_rhs_vjp(self.h, _ptr(x), _ptr(kbar), _ptr(xbar)))

    def limit_vjp(self, z, ybar, zbar):
        self._chk(self._L.rkdg_limit_vjp(self.h, _ptr(z), _ptr(ybar), _ptr(zbar)))

    def step_vjp(self, x, dt: float, xbar):
        self._chk(self._L.rkdg_step_vjp(self.h, _ptr(x), dt, _ptr(xbar)))

    def adjoint_run(self, x0, nsteps: int, dt: float, checkpoint_every: int, xbar, xT=None):
        self._chk(self._L.rkdg_adjoint_run(self.h, _ptr(x0), nsteps, dt, checkpoint_every,
                                           _ptr(xbar), _ptr(xT) if xT is not None else None))

    # -- batched independent problems -----------------------------------------
    def batch_setup(self, elem_offsets, gammas, covolumes):
        off = np.ascontiguousarray(elem_offsets, dtype=np.int32)
        g = np.ascontiguousarray(gammas, dtype=np.float64)
        b = np.ascontiguousarray(covolumes, dtype=np.float64)
        self.nprob = len(g)
        self._chk(self._L.rkdg_batch_setup(self.h, self.nprob, off.ctypes.data_as(_capi._ip),
                                           g.ctypes.data_as(_capi._dp), b.ctypes.data_as(_capi._dp)))

    def batch_run(self, x, t_end: float, cfl: float = 0.3, dt0: float = 0.0, dt_mode: int = 0,
                  max_steps: int = 0, use_graph: bool = True, limit_initial: bool = True) -> dict:
        np_ = self.nprob
        self._initial_limit(limit_initial)
        steps = np.zeros(np_, np.int32)
        t = np.zeros(np_)
        sdt = np.zeros(np_)
        self._chk(self._L.rkdg_batch_run(self.h, _ptr(x), t_end, cfl, dt0, dt_mode, max_steps,
                                         int(use_graph), steps.ctypes.data_as(_capi._ip),
                                         t.ctypes.data_as(_capi._dp), sdt.ctypes.data_as(_capi._dp)))
        return {"steps": steps, "t": t, "sum_dt": sdt}


# ---- reference-named mirrors -------------------------------------------------
class FE_Evolution:
    """TimeDependentOperator for the DG right-hand side (fe_evolution.hpp:27-82).
    ``Mult(x, y)`` fills y and returns (and stores) max_char_speed."""

    def __init__(self, ctx: Context):
        self.ctx = ctx
        self.max_char_speed = 0.0

    def Mult(self, x, y) -> float:
        self.max_char_speed = self.ctx.rhs(x, y)
        return self.max_char_speed


class Averager:
    """Cell means (averager.hpp:139-152): ``avgs[iEq * NE + e]``."""

    def __init__(self, ctx: Context):
        self.ctx = ctx
        import torch
        self.avgs = torch.zeros(ctx.neq * ctx.ne, dtype=torch.float64, device="cuda")

    def computeMeanValues(self, x):
        self.ctx.cell_means(x, self.avgs)

    def readElementAverageByNumber(self, iCell: int):
        return self.avgs.view(self.ctx.neq, self.ctx.ne)[:, iCell].cpu().numpy()


class Indicator:
    code = IND_NOWHERE

    def __init__(self, function: int = FUN_MICHALAK):
        self.function = function


class IndicatorNowhere(Indicator):
    code = IND_NOWHERE


class IndicatorEverywhere(Indicator):
    code = IND_EVERYWHERE


class IndicatorBJ(Indicator):
    """BJ-family indicator; ``function`` selects classical BJ,
    Venkatakrishnan or Michalak (the shipped code computes Michalak,
    indicator_bj.cpp:76-79)."""
    code = IND_BJ


class Limiter:
    code = LIM_FINDIFF

    def __init__(self, ctx: Context, indicator: Indicator, haveLastHope: bool = True,
                 quirks: int = 0):
        self.ctx = ctx
        self.indicator = indicator
        ctx.set_limiter(self.code, indicator.code, indicator.function, int(haveLastHope), quirks)

    def update(self, x):
        self.ctx.limit(x)


class LimiterFinDiff(Limiter):
    code = LIM_FINDIFF


class LimiterMultiplier(Limiter):
    code = LIM_MULTI


class ExplicitRKLimitedSolver:
    """Butcher-form RK with a limiter after every stage
    (rk_explicit_limited.hpp:24-60).  ``Step`` does not advance t."""

    def __init__(self, s: int, a, b, c, limiter: Limiter):
        self.s, self.a, self.b, self.c = s, list(a), list(b), list(c)
        self.limiter = limiter
        self.f = None

    def Init(self, f: FE_Evolution):
        self.f = f
        f.ctx.set_tableau(self.s, self.a, self.b, self.c)

    def Step(self, x, t: float, dt: float) -> float:
        mcs = self.f.ctx.step(x, dt)
        self.f.max_char_speed = mcs
        return mcs
