"""The MFEM adapter (rkdg3d_gb300/adapters/mfem) compiles against MFEM's
interface -- here the test-only stand-in oracle/refshim/mfem.hpp, MFEM itself
is not installed -- and links against the library's C ABI with no
unresolved symbol.  The adapter's classes replace FE_Evolution,
ExplicitRKLimitedSolver and Limiter::update in the reference's main.cpp."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ADAPTER = os.path.join(ROOT, "rkdg3d_gb300", "adapters", "mfem", "rkdg_mfem.cpp")
CUDA_INC = "/usr/local/cuda/include"
CUDA_LIB = "/usr/local/cuda/lib64"


def _gxx():
    gxx = shutil.which("g++")
    if not gxx or not os.path.isdir(CUDA_INC):
        pytest.skip("g++ or the CUDA headers not available")
    return gxx


def test_adapter_compiles_and_links(tmp_path):
    gxx = _gxx()
    obj = str(tmp_path / "rkdg_mfem.o")
    flags = ["-std=c++17", "-Wall", "-Werror", "-fPIC", "-I", os.path.join(ROOT, "oracle", "refshim"),
             "-I", os.path.join(ROOT, "include"), "-I", CUDA_INC]
    r = subprocess.run([gxx, *flags, "-c", ADAPTER, "-o", obj], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    from rkdg3d_gb300 import buildlib
    lib = buildlib.lib_path()
    if not os.path.exists(lib):
        pytest.skip("library not built")
    out = str(tmp_path / "libadapter.so")
    r = subprocess.run([gxx, "-shared", obj, "-o", out, "-L", os.path.dirname(lib), "-lrkdg_gb300",
                        "-L", CUDA_LIB, "-lcudart", "-Wl,--no-undefined"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
