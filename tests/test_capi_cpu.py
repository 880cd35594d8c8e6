"""CPU tests of the product library boundary: it builds, loads, exports every
entry point declared in include/rkdg_gpu.h, and fails loudly (no fallback)
when no device is present.  No compute call is made here."""
import ctypes as C
import os
import re

import pytest

from rkdg3d_gb300 import _capi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "rkdg_gpu.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(rkdg_[a-z0-9_]+)\s*\(", text)))


def test_library_built_and_loads():
    assert os.path.exists(_capi.lib_path()), "run __graft_entry__.build() first"
    _capi.load()


def test_exports_every_declared_symbol():
    L = C.CDLL(_capi.lib_path())
    names = declared_functions()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    assert sorted(_capi.EXPORTED) == names


def test_create_without_device_fails_loudly():
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a device is present")
    L = _capi.load()
    h = C.c_void_p()
    assert L.rkdg_create(C.byref(h), 0) == 8  # RKDG_ERR_NOT_FOUND
    assert not h.value


def test_context_construction_raises_without_device():
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a device is present")
    from rkdg3d_gb300 import mesh as M
    from rkdg3d_gb300.solver import Context, RkdgError
    with pytest.raises(RkdgError):
        Context(M.quad_grid(4, 2), 1)


def test_null_context_rejected():
    L = _capi.load()
    assert L.rkdg_set_physics(None, 0, 0, 1.4, 0.0, 1.0) == 1
    assert L.rkdg_rhs(None, None, None, None) == 1
    assert L.rkdg_kernel_launches(None) == -1
