"""Build the GB300 RKDG shared library (librkdg_gb300.so) in-tree.

Compiles every translation unit under ``csrc/`` with nvcc for sm_103a only
(``-gencode arch=compute_103a,code=sm_103a``) in parallel and links one
shared library with a plain C ABI (``include/rkdg_gpu.h``).  No torch types
cross the boundary.
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(ROOT, "include")
OBJDIR = os.path.join(HERE, "_build")
LIBDIR = os.path.join(HERE, "_lib")
LIBNAME = "librkdg_gb300.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc_path() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build rkdg3d_gb300")


def lib_path() -> str:
    return os.path.join(LIBDIR, LIBNAME)


def _sources():
    return sorted(f for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))


def _headers_digest() -> str:
    h = hashlib.sha1()
    for d in (CSRC, INCLUDE):
        for f in sorted(os.listdir(d)):
            if f.endswith((".h", ".cuh")):
                with open(os.path.join(d, f), "rb") as fh:
                    h.update(f.encode() + fh.read())
    return h.hexdigest()


def _compile(nvcc: str, src: str, flags) -> str:
    obj = os.path.join(OBJDIR, src + ".o")
    # -ftz=true: FP32 arithmetic flushes subnormals (below 1.2e-38) to zero,
    # which drops the subnormal fix-ups of the reciprocal / square-root
    # approximations; the FP32-bulk path never carries values that small
    cmd = [nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-ftz=true", "-Xcompiler", "-fPIC",
           "-I", INCLUDE, "-I", CSRC, *flags, "-c", os.path.join(CSRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
    return obj


def build(verbose: bool = False, force: bool = False, extra_flags=()) -> str:
    """Compile and link; returns the library path.  Incremental on sources."""
    nvcc = nvcc_path()
    os.makedirs(OBJDIR, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    stamp = os.path.join(OBJDIR, "headers.sha1")
    digest = _headers_digest() + "|" + " ".join(extra_flags)
    if not force and os.path.exists(stamp):
        with open(stamp) as fh:
            force = fh.read() != digest
    else:
        force = True
    srcs = _sources()
    todo = []
    for s in srcs:
        obj = os.path.join(OBJDIR, s + ".o")
        if force or not os.path.exists(obj) or os.path.getmtime(obj) < os.path.getmtime(os.path.join(CSRC, s)):
            todo.append(s)
    workers = max(1, min(len(todo), os.cpu_count() or 4))
    with cf.ThreadPoolExecutor(max_workers=workers) as ex:
        for obj in ex.map(lambda s: _compile(nvcc, s, list(extra_flags)), todo):
            if verbose:
                print("compiled", obj, file=sys.stderr)
    objs = [os.path.join(OBJDIR, s + ".o") for s in srcs]
    out = lib_path()
    tmp = out + ".tmp"
    cmd = [nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, out)
    with open(stamp, "w") as fh:
        fh.write(digest)
    return out


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))
