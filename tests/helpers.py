"""Shared test helpers: matched (oracle, device context) pairs on one case."""
from __future__ import annotations

import numpy as np

from rkdg3d_gb300 import cases
from rkdg3d_gb300 import mesh as M


def random_state(coords: np.ndarray, gamma=1.4, b=0.0, seed=0, amp=0.15, vel=0.3):
    """Random physical nodal state (smooth background + nodal noise)."""
    rng = np.random.default_rng(seed)
    dim, n = coords.shape
    rho = 1.0 + amp * rng.uniform(-1, 1, n) + 0.1 * np.sin(2 * np.pi * coords[0])
    p = 1.0 + amp * rng.uniform(-1, 1, n)
    vels = [vel * rng.uniform(-1, 1, n) for _ in range(dim)]
    return cases.conservative([rho, *vels, p], gamma, b)


def rel_l1(a, b):
    return float(np.abs(a - b).sum() / max(np.abs(b).sum(), 1e-300))


def periodic_case(geom, n, order, rsolver, averaging=0, gamma=1.4, covolume=0.0):
    if geom == M.GEOM_CUBE:
        mesh = M.hex_grid(n, n, n)
    elif geom == M.GEOM_SQUARE:
        mesh = M.quad_grid(n, n, 0, 1, 0, 1, periodic=(True, True))
    else:
        raise ValueError(geom)
    return cases.Case("periodic", mesh, order, rsolver, averaging, gamma=gamma, covolume=covolume)


def walled_case(geom, n, order, rsolver, averaging=0, gamma=1.4, covolume=0.0, bc=0):
    """Closed box with boundary type ``bc`` on every side."""
    if geom == M.GEOM_CUBE:
        mesh = M.hex_grid(n, n, n, periodic=(False, False, False))
        attrs = range(1, 7)
    elif geom == M.GEOM_SQUARE:
        mesh = M.quad_grid(n, n + 1, 0, 1, 0, 0.7)
        attrs = range(1, 5)
    else:
        mesh = M.tri_grid(n, n, 0, 1, 0, 1, jitter=0.2, seed=3)
        attrs = range(1, 5)
    return cases.Case("walled", mesh, order, rsolver, averaging, gamma=gamma, covolume=covolume,
                      bcs=[(a, bc, None) for a in attrs])
