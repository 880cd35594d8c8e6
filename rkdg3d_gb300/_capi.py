"""ctypes binding of ``librkdg_gb300.so`` (C ABI declared in include/rkdg_gpu.h).

The library is built in-tree by ``rkdg3d_gb300.build``.  There is no
fallback: if the shared library is missing or cannot be loaded, every entry
point raises.
"""
from __future__ import annotations

import ctypes as C
import os

from . import buildlib as _build

_lib = None

_vp = C.c_void_p
_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)

# (name, restype, argtypes)
_SIGS = [
    ("rkdg_create", C.c_int, [C.POINTER(C.c_void_p), C.c_int]),
    ("rkdg_destroy", C.c_int, [_vp]),
    ("rkdg_last_error", C.c_char_p, [_vp, C.POINTER(C.c_longlong)]),
    ("rkdg_set_stream", C.c_int, [_vp, _vp]),
    ("rkdg_synchronize", C.c_int, [_vp]),
    ("rkdg_set_physics", C.c_int, [_vp, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double]),
    ("rkdg_upload_mesh", C.c_int, [_vp, _vp]),
    ("rkdg_set_bc", C.c_int, [_vp, C.c_int, C.c_int, _dp]),
    ("rkdg_set_limiter", C.c_int, [_vp, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int]),
    ("rkdg_set_tableau", C.c_int, [_vp, C.c_int, _dp, _dp, _dp]),
    ("rkdg_set_precision", C.c_int, [_vp, C.c_int]),
    ("rkdg_set_tuning", C.c_int, [_vp, C.c_int, C.c_int]),
    ("rkdg_set_solver_quirks", C.c_int, [_vp, C.c_int]),
    ("rkdg_sizes", C.c_int, [_vp, C.POINTER(C.c_longlong), _ip, _ip]),
    ("rkdg_node_coords_host", C.c_int, [_vp, _dp]),
    ("rkdg_hmin", C.c_int, [_vp, _dp]),
    ("rkdg_rhs", C.c_int, [_vp, _vp, _vp, _dp]),
    ("rkdg_face_speed", C.c_int, [_vp, _vp, _dp]),
    ("rkdg_limit", C.c_int, [_vp, _vp]),
    ("rkdg_cell_means", C.c_int, [_vp, _vp, _vp]),
    ("rkdg_step", C.c_int, [_vp, _vp, C.c_double, _dp]),
    ("rkdg_run", C.c_int, [_vp, _vp, C.c_double, C.c_double, C.c_double, C.c_int, C.c_int,
                           _ip, _dp, _dp, _dp]),
    ("rkdg_run_continue", C.c_int, [_vp, _vp, C.c_double, C.c_double, C.c_double, C.c_double,
                                    C.c_int, C.c_int, _ip, _dp, _dp, _dp]),
    ("rkdg_totals", C.c_int, [_vp, _vp, _dp]),
    ("rkdg_riemann_batch", C.c_int, [_vp, C.c_int, _vp, _vp, _vp, _vp, _vp]),
    ("rkdg_batch_setup", C.c_int, [_vp, C.c_int, _ip, _dp, _dp]),
    ("rkdg_batch_run", C.c_int, [_vp, _vp, C.c_double, C.c_double, C.c_double, C.c_int, C.c_int,
                                 C.c_int, _ip, _dp, _dp]),
    ("rkdg_rhs_vjp", C.c_int, [_vp, _vp, _vp, _vp]),
    ("rkdg_limit_vjp", C.c_int, [_vp, _vp, _vp, _vp]),
    ("rkdg_step_vjp", C.c_int, [_vp, _vp, C.c_double, _vp]),
    ("rkdg_adjoint_run", C.c_int, [_vp, _vp, C.c_int, C.c_double, C.c_int, _vp, _vp]),
    ("rkdg_kernel_launches", C.c_longlong, [_vp]),
    ("rkdg_limit_static", C.c_int, [_vp, _vp]),
    ("rkdg_autotune", C.c_int, [_vp, _vp, _ip, _ip, _ip]),
]

EXPORTED = [s[0] for s in _SIGS]


class MeshDesc(C.Structure):
    _fields_ = [("dim", C.c_int), ("geom", C.c_int), ("order", C.c_int),
                ("num_elements", C.c_int), ("elem_vertices", _ip), ("elem_coords", _dp),
                ("num_bdr", C.c_int), ("bdr_vertices", _ip), ("bdr_attr", _ip)]


def lib_path() -> str:
    return _build.lib_path()


def load(build_if_missing: bool = False):
    """Load the CUDA library.  Raises if it is absent (no CPU fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    path = lib_path()
    if not os.path.exists(path):
        if not build_if_missing:
            raise RuntimeError(
                f"rkdg3d_gb300 CUDA library not built ({path}); run "
                "`python -c 'import __graft_entry__ as g; g.build()'`")
        _build.build()
    L = C.CDLL(path)
    for name, res, args in _SIGS:
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L
