"""ctypes binding of oracle/_ref/librefpin.so: the reference's own pointwise
sources (physics/physics.cpp, riemannsolvers/rs_*.cpp and the boundary
ghost-state files bc/boundary_integrator_*.cpp) compiled unmodified against a
test-only MFEM stand-in (oracle/refshim).

TEST INFRASTRUCTURE ONLY.  It needs the reference source tree to build
(``make -C oracle ref``), so it exists where that tree exists; the committed
vectors it produced (tests/golden/refpin.npz, written by
tests/golden/make_refpin.py) carry its results to hosts without it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_ref", "librefpin.so")
REFERENCE = os.environ.get("RKDG_REFERENCE_TREE", "/root/reference")

_dp = C.POINTER(C.c_double)
_lib = None


def available() -> bool:
    """True when the library exists or can be built from the reference tree."""
    return os.path.exists(LIB) or os.path.isdir(os.path.join(REFERENCE, "src", "physics"))


def build() -> str:
    if not os.path.exists(LIB):
        subprocess.run(["make", "-C", HERE, "-s", "ref", f"REF={REFERENCE}"], check=True)
    return LIB


def lib():
    global _lib
    if _lib is None:
        L = C.CDLL(build())
        L.pin_set_physics.argtypes = [C.c_double, C.c_double, C.c_double, C.c_int]
        L.pin_eos.argtypes = [C.c_int, C.c_int, _dp, _dp]
        L.pin_flux.argtypes = [C.c_int, C.c_int, _dp, _dp]
        L.pin_speeds.argtypes = [C.c_int, C.c_int, C.c_int, _dp, _dp, _dp, _dp]
        L.pin_riemann.argtypes = [C.c_int, C.c_int, C.c_int, _dp, _dp, _dp, _dp, _dp]
        L.pin_right_state.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, _dp, _dp, C.c_double,
                                      _dp, _dp, _dp]
        _lib = L
    return _lib


def _d(a):
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_dp)


def _c(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def set_physics(gamma: float, covolume: float, gas_constant: float, dim: int) -> None:
    lib().pin_set_physics(gamma, covolume, gas_constant, dim + 2)


def eos(u, dim):
    """[n][6]: pressure, sound speed, max char speed, Mach, StateIsPhysical, T."""
    u = _c(u)
    out = np.zeros((u.shape[0], 6))
    lib().pin_eos(u.shape[0], dim, _d(u), _d(out))
    return out


def flux(u, dim):
    u = _c(u)
    out = np.zeros((u.shape[0], dim + 2, dim))
    lib().pin_flux(u.shape[0], dim, _d(u), _d(out))
    return out


def speeds(kind, u1, u2, nor):
    """kind 0 TRRS, 1 Einfeldt, of the two states rotated into nor's frame."""
    u1, u2, nor = _c(u1), _c(u2), _c(nor)
    dim = nor.shape[1]
    out = np.zeros_like(u1)
    lib().pin_speeds(kind, u1.shape[0], dim, _d(u1), _d(u2), _d(nor), _d(out))
    return out


def riemann(rs, u1, u2, nor):
    u1, u2, nor = _c(u1), _c(u2), _c(nor)
    dim = nor.shape[1]
    f = np.zeros_like(u1)
    sp = np.zeros(u1.shape[0])
    if lib().pin_riemann(rs, u1.shape[0], dim, _d(u1), _d(u2), _d(nor), _d(f), _d(sp)):
        raise ValueError("unknown Riemann solver")
    return f, sp


def right_state(bc, s1, nor, prm=None, s2_in=None, nor_pad=0.0, rs=3):
    s1, nor = _c(s1), _c(nor)
    dim = nor.shape[1]
    prm = None if prm is None else _c(np.pad(np.ravel(prm), (0, max(0, dim + 2 - np.size(prm)))))
    s2_in = None if s2_in is None else _c(s2_in)
    out = np.zeros_like(s1)
    if lib().pin_right_state(bc, rs, s1.shape[0], dim, _d(s1), _d(nor), nor_pad, _d(prm),
                             _d(s2_in), _d(out)):
        raise ValueError("unknown boundary condition")
    return out
