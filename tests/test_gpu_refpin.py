"""Device Riemann solvers against vectors the REFERENCE'S own code produced.

tests/golden/refpin.npz was written by the reference's riemannsolvers/rs_*.cpp
and physics/physics.cpp compiled unmodified (tests/golden/make_refpin.py).
The FP64 device solvers (rkdg_riemann_batch, the same device functions the
face kernels call) must give the same -1 (non-physical) pattern and fluxes
and speeds within 1e-12 relative: they form the TRRS powers as
exp2(e * log2(a)), which differs from pow in the last bits.
"""
import os

import numpy as np
import pytest
import torch

from rkdg3d_gb300 import mesh as M
from rkdg3d_gb300.solver import (AVG_TRRS, Context, Physics, RiemannSolverHLL, RiemannSolverHLLC,
                                 RiemannSolverLLF, RiemannSolverRusanov)
from tests.golden.make_refpin import EOS

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(__file__), "golden", "refpin.npz")
KEYS = [(dim, e) for dim in (2, 3) for e in EOS]


def dev(x):
    return torch.tensor(np.ascontiguousarray(x), dtype=torch.float64, device="cuda:0")


@pytest.mark.parametrize("rs", [0, 1, 2, 3], ids=["rusanov", "llf", "hll", "hllc"])
@pytest.mark.parametrize("dim,eos", KEYS, ids=[f"d{d}-{e[0]}" for d, e in KEYS])
def test_device_riemann_matches_reference(cuda, dim, eos, rs):
    g = np.load(GOLD)
    key = f"d{dim}/{eos[0]}"
    _, gamma, b, R = eos
    mesh = M.hex_grid(3, 3, 3) if dim == 3 else M.quad_grid(3, 3, 0, 1, 0, 1, periodic=(True, True))
    ctx = Context(mesh, 1, device=0)
    solver = (RiemannSolverRusanov, RiemannSolverLLF, RiemannSolverHLL, RiemannSolverHLLC)[rs]
    ctx.set_physics(solver(AVG_TRRS), Physics(gamma, b, R))
    u1, u2, nor = g[f"{key}/u1"], g[f"{key}/u2"], g[f"{key}/nor"]
    n, neq = u1.shape
    flux = torch.zeros((n, neq), dtype=torch.float64, device="cuda")
    sp = torch.zeros(n, dtype=torch.float64, device="cuda")
    ctx.riemann_batch(dev(u1), dev(u2), dev(nor), flux, sp)
    f, s = flux.cpu().numpy(), sp.cpu().numpy()
    ref_f, ref_s = g[f"{key}/rs{rs}/flux"], g[f"{key}/rs{rs}/speed"]
    assert np.array_equal(s == -1.0, ref_s == -1.0)
    ok = ref_s != -1.0
    assert np.allclose(s[ok], ref_s[ok], rtol=1e-12, atol=1e-14)
    scale = np.abs(ref_f[ok]).max(axis=1, keepdims=True) + 1e-300
    assert (np.abs(f[ok] - ref_f[ok]) / scale).max() < 1e-12
