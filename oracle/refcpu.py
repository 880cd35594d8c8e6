"""ctypes binding of the CPU FP64 oracle (refcpu).

TEST INFRASTRUCTURE ONLY: imported by tests/, ``__graft_entry__.smoke()`` and
the CPU-baseline / reference legs of ``bench.py``.  The product package
(rkdg3d_gb300) never imports this module.  Parity is unpinned at the MFEM
boundary; see refcpu.h.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "librefcpu.so")

_lib = None

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (g++, portable flags)."""
    src = os.path.join(HERE, "refcpu.cpp")
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(src):
        subprocess.run(["make", "-C", HERE, "-s"], check=True)
    return LIB


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB)
        L.ref_create.restype = C.c_void_p
        L.ref_create.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, _ip, _dp, C.c_int, _ip, _ip]
        L.ref_destroy.argtypes = [C.c_void_p]
        L.ref_set_physics.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double]
        L.ref_set_bc.argtypes = [C.c_void_p, C.c_int, C.c_int, _dp]
        L.ref_right_state.argtypes = [C.c_void_p, C.c_int, _dp, _dp, _dp]
        L.ref_set_limiter.argtypes = [C.c_void_p] + [C.c_int] * 5
        L.ref_set_tableau.argtypes = [C.c_void_p, C.c_int, _dp, _dp, _dp]
        L.ref_set_threads.argtypes = [C.c_int]
        L.ref_set_solver_quirks.argtypes = [C.c_void_p, C.c_int]
        L.ref_ndofs.restype = C.c_longlong
        L.ref_ndofs.argtypes = [C.c_void_p]
        L.ref_nd.argtypes = [C.c_void_p]
        L.ref_neq.argtypes = [C.c_void_p]
        L.ref_nfaces.argtypes = [C.c_void_p, _ip, _ip]
        L.ref_node_coords.argtypes = [C.c_void_p, _dp]
        L.ref_hmin.restype = C.c_double
        L.ref_hmin.argtypes = [C.c_void_p]
        L.ref_rhs.argtypes = [C.c_void_p, _dp, _dp, _dp]
        L.ref_face_speed.argtypes = [C.c_void_p, _dp, _dp]
        L.ref_means.argtypes = [C.c_void_p, _dp, _dp]
        L.ref_limit.argtypes = [C.c_void_p, _dp]
        L.ref_step.argtypes = [C.c_void_p, _dp, C.c_double, _dp]
        L.ref_run.argtypes = [C.c_void_p, _dp, C.c_double, C.c_double, C.c_double, C.c_int, C.c_int,
                              _ip, _dp, _dp, _dp]
        L.ref_run_continue.argtypes = [C.c_void_p, _dp, C.c_double, C.c_double, C.c_double,
                                       C.c_double, C.c_int, C.c_int, _ip, _dp, _dp, _dp]
        L.ref_totals.argtypes = [C.c_void_p, _dp, _dp]
        L.ref_total_energy.restype = C.c_double
        L.ref_total_energy.argtypes = [C.c_void_p, _dp]
        L.ref_riemann.argtypes = [C.c_void_p, C.c_int, _dp, _dp, _dp, _dp, _dp]
        L.ref_pointwise.argtypes = [C.c_void_p, C.c_int, C.c_int, _dp, _dp, _dp, _dp]
        L.ref_last_error.restype = C.c_char_p
        L.ref_last_error.argtypes = [C.c_void_p]
        _lib = L
    return _lib


def _d(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_dp)


def _i(a: np.ndarray):
    assert a.dtype == np.int32 and a.flags.c_contiguous
    return a.ctypes.data_as(_ip)


class OracleError(RuntimeError):
    pass


class Oracle:
    """One reference-semantics CPU solver on one mesh."""

    def __init__(self, mesh, order: int):
        L = lib()
        m = mesh.contiguous()
        self._mesh = m
        self.h = L.ref_create(m.dim, m.geom, order, m.num_elements, _i(m.elem_vertices),
                              _d(m.elem_coords), m.bdr_vertices.shape[0], _i(m.bdr_vertices),
                              _i(m.bdr_attr))
        if not self.h:
            raise OracleError("ref_create failed (unsupported element/order or invalid mesh)")
        self.dim = m.dim
        self.order = order
        self.ndofs = int(L.ref_ndofs(self.h))
        self.nd = int(L.ref_nd(self.h))
        self.neq = int(L.ref_neq(self.h))
        self.ne = m.num_elements

    def __del__(self):
        if getattr(self, "h", None):
            lib().ref_destroy(self.h)
            self.h = None

    def _chk(self, st):
        if st != 0:
            raise OracleError(f"oracle status {st}: {lib().ref_last_error(self.h).decode()}")

    @property
    def n(self) -> int:
        return self.ndofs * self.neq

    def set_physics(self, rsolver=0, averaging=0, gamma=1.4, covolume=0.0, gas_constant=1.0):
        self._chk(lib().ref_set_physics(self.h, rsolver, averaging, gamma, covolume, gas_constant))

    def set_bc(self, attr, bctype, state=None):
        """state: conservative variables, or the boundary condition's
        parameters in its first entries; padded to five values."""
        st = None
        if state is not None:
            st = np.zeros(5, dtype=np.float64)
            v = np.asarray(state, dtype=np.float64).ravel()
            st[:v.size] = v
        self._chk(lib().ref_set_bc(self.h, attr, bctype, _d(st) if st is not None else None))

    def right_state(self, attr, s1, nor):
        s1 = np.ascontiguousarray(s1, dtype=np.float64)
        nor = np.ascontiguousarray(nor, dtype=np.float64)
        s2 = np.zeros_like(s1)
        self._chk(lib().ref_right_state(self.h, attr, _d(s1), _d(nor), _d(s2)))
        return s2

    def set_limiter(self, limiter=0, indicator=0, function=2, last_hope=1, quirks=0):
        self._chk(lib().ref_set_limiter(self.h, limiter, indicator, function, last_hope, quirks))

    def set_solver_quirks(self, flags):
        self._chk(lib().ref_set_solver_quirks(self.h, int(flags)))
        self._solver_quirks = int(flags)

    def set_tableau(self, s, a, b, c):
        a = np.ascontiguousarray(a if len(a) else [0.0], dtype=np.float64)
        b = np.ascontiguousarray(b, dtype=np.float64)
        c = np.ascontiguousarray(c if len(c) else [0.0], dtype=np.float64)
        self._chk(lib().ref_set_tableau(self.h, s, _d(a), _d(b), _d(c)))

    def node_coords(self) -> np.ndarray:
        out = np.zeros(self.dim * self.ndofs)
        self._chk(lib().ref_node_coords(self.h, _d(out)))
        return out.reshape(self.dim, self.ndofs)

    def hmin(self) -> float:
        return float(lib().ref_hmin(self.h))

    def nfaces(self):
        a = C.c_int()
        b = C.c_int()
        lib().ref_nfaces(self.h, C.byref(a), C.byref(b))
        return a.value, b.value

    def rhs(self, x: np.ndarray):
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.zeros_like(x)
        m = C.c_double()
        self._chk(lib().ref_rhs(self.h, _d(x), _d(y), C.byref(m)))
        return y, m.value

    def face_speed(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        m = C.c_double()
        self._chk(lib().ref_face_speed(self.h, _d(x), C.byref(m)))
        return m.value

    def means(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        out = np.zeros(self.neq * self.ne)
        self._chk(lib().ref_means(self.h, _d(x), _d(out)))
        return out

    def limit(self, x):
        x = np.array(x, dtype=np.float64, copy=True)
        self._chk(lib().ref_limit(self.h, _d(x)))
        return x

    def step(self, x, dt):
        x = np.array(x, dtype=np.float64, copy=True)
        m = C.c_double()
        self._chk(lib().ref_step(self.h, _d(x), dt, C.byref(m)))
        return x, m.value

    def run(self, x, t_end, cfl=0.3, dt0=0.0, dt_mode=0, max_steps=0, limit_initial=True):
        """ref_run; limit_initial limits x once first (main.cpp:264-265)."""
        q = getattr(self, "_solver_quirks", 0)
        want = (q & ~2) | (0 if limit_initial else 2)
        if want != q:
            self.set_solver_quirks(want)
        x = np.array(x, dtype=np.float64, copy=True)
        steps = C.c_int()
        t = C.c_double()
        dt = C.c_double()
        sdt = C.c_double()
        self._chk(lib().ref_run(self.h, _d(x), t_end, cfl, dt0, dt_mode, max_steps, C.byref(steps),
                                C.byref(t), C.byref(dt), C.byref(sdt)))
        return x, {"steps": steps.value, "t": t.value, "dt": dt.value, "sum_dt": sdt.value}

    def run_continue(self, x, t0, dt, t_end, cfl=0.3, dt_mode=0, max_steps=0):
        """ref_run_continue: the loop from time t0 with the next dt known
        (the reference's restart, main.cpp:461-490)."""
        x = np.array(x, dtype=np.float64, copy=True)
        steps = C.c_int()
        t = C.c_double()
        dto = C.c_double()
        sdt = C.c_double()
        self._chk(lib().ref_run_continue(self.h, _d(x), t0, dt, t_end, cfl, dt_mode, max_steps,
                                         C.byref(steps), C.byref(t), C.byref(dto), C.byref(sdt)))
        return x, {"steps": steps.value, "t": t.value, "dt": dto.value, "sum_dt": sdt.value}

    def totals(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        out = np.zeros(self.neq)
        self._chk(lib().ref_totals(self.h, _d(x), _d(out)))
        return out

    def total_energy(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        return float(lib().ref_total_energy(self.h, _d(x)))

    def pointwise(self, what, u1, u2=None, nor=None):
        """ref_pointwise: what 0 EoS [n][4] (p, c, max speed, physical),
        1 flux [n][neq][dim], 2 TRRS / 3 Einfeldt speeds [n][neq] of u1, u2
        rotated into nor's frame."""
        u1 = np.ascontiguousarray(u1, dtype=np.float64)
        n = u1.shape[0]
        u2 = None if u2 is None else np.ascontiguousarray(u2, dtype=np.float64)
        nor = None if nor is None else np.ascontiguousarray(nor, dtype=np.float64)
        width = {0: 4, 1: self.neq * self.dim, 2: self.neq, 3: self.neq}[what]
        out = np.zeros((n, width))
        self._chk(lib().ref_pointwise(self.h, what, n, _d(u1), None if u2 is None else _d(u2),
                                      None if nor is None else _d(nor), _d(out)))
        return out

    def riemann(self, u1, u2, nor):
        u1 = np.ascontiguousarray(u1, dtype=np.float64)
        u2 = np.ascontiguousarray(u2, dtype=np.float64)
        nor = np.ascontiguousarray(nor, dtype=np.float64)
        n = u1.shape[0]
        flux = np.zeros_like(u1)
        sp = np.zeros(n)
        lib().ref_riemann(self.h, n, _d(u1), _d(u2), _d(nor), _d(flux), _d(sp))
        return flux, sp


def set_threads(n: int) -> None:
    lib().ref_set_threads(int(n))
