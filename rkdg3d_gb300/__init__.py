"""rkdg3d_gb300 — GB300-native (sm_103a) RKDG hot path for RKDG3D.

The compute path is the CUDA shared library ``librkdg_gb300.so`` behind the C
ABI in ``include/rkdg_gpu.h``; this package holds its in-tree build, the
ctypes binding, the reference-named host mirror (:mod:`.solver`) and the
host-side mesh / case set-up (:mod:`.mesh`, :mod:`.cases`).
"""
from . import mesh  # noqa: F401
from .buildlib import build, lib_path  # noqa: F401

__all__ = ["mesh", "build", "lib_path"]
