"""Write tests/golden/refpin.npz: golden vectors produced by the REFERENCE'S
OWN pointwise code.

The reference's physics/physics.cpp, riemannsolvers/rs_*.cpp and the
boundary ghost-state files bc/boundary_integrator_*.cpp are compiled
unmodified against a test-only MFEM stand-in (oracle/refshim, ``make -C
oracle ref``); this script calls them (through oracle/refpin.py) on seeded
inputs and stores inputs and outputs.  tests/test_refpin.py checks the
oracle against these vectors on every CPU run, re-derives them from the
reference library where the reference tree exists, and the GPU tests check
the device Riemann solvers against them.

    python tests/golden/make_refpin.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import refpin  # noqa: E402

OUT = os.path.join(HERE, "refpin.npz")
# (name, gamma, covolume, gas constant)
EOS = (("perfect", 1.4, 0.0, 1.0), ("covolume", 1.4, 0.01, 0.7))
N_RANDOM = 96


def conservative(rho, u, p, gamma, b):
    e = p * (1.0 - rho * b) / (gamma - 1.0) + 0.5 * rho * np.sum(u * u, axis=1)
    return np.column_stack([rho, rho[:, None] * u, e])


def unit(v):
    return v / np.linalg.norm(v, axis=1, keepdims=True)


def states(rng, n, dim, gamma, b, vmax):
    rho = rng.uniform(0.1, 2.0, n)
    u = rng.uniform(-vmax, vmax, (n, dim))
    p = rng.uniform(0.05, 3.0, n)
    return conservative(rho, u, p, gamma, b)


def inputs(dim, gamma, b, seed):
    """Left/right states and unit normals: subsonic and supersonic pairs
    (every HLL / HLLC branch), near-vacuum states, axis normals (the 3D
    rotation's degenerate branch at |cos psi| <= 1e-6) and non-physical
    states (negative density, negative energy, negative pressure)."""
    rng = np.random.default_rng(seed)
    n = N_RANDOM
    u1 = np.concatenate([states(rng, n, dim, gamma, b, 0.6), states(rng, n // 2, dim, gamma, b, 5.0)])
    u2 = np.concatenate([states(rng, n, dim, gamma, b, 0.6), states(rng, n // 2, dim, gamma, b, 5.0)])
    nor = unit(rng.normal(size=(u1.shape[0], dim)))
    # axis normals, both signs
    axes = np.concatenate([np.eye(dim), -np.eye(dim)])
    k = axes.shape[0]
    nor[:k] = axes
    nor[k:2 * k] = axes
    # near-vacuum states on one side
    vac = conservative(np.full(8, 1e-5), rng.uniform(-0.1, 0.1, (8, dim)), np.full(8, 1e-6), gamma, b)
    u1[2 * k:2 * k + 8] = vac
    # non-physical states
    bad = u1[2 * k + 8:2 * k + 12].copy()
    bad[0, 0] = -0.1                       # negative density
    bad[1, -1] = -0.2                      # negative energy
    bad[2, 1] = 6.0 * np.sqrt(bad[2, 0] * bad[2, -1])  # kinetic energy above E: p < 0
    bad[3, 0] = -1e-3
    u1[2 * k + 8:2 * k + 12] = bad
    u2[2 * k + 20] = bad[1]
    return u1, u2, nor


def bc_inputs(dim, gamma, b, seed):
    rng = np.random.default_rng(seed)
    n = 64
    s1 = states(rng, n, dim, gamma, b, 0.8)
    nor = unit(rng.normal(size=(n, dim)))
    nor[:2 * dim] = np.concatenate([np.eye(dim), -np.eye(dim)])
    outer = states(rng, 1, dim, gamma, b, 0.5)[0]
    return s1, nor, outer


def main():
    data = {}
    for di, dim in enumerate((2, 3)):
        for ei, (ename, gamma, b, R) in enumerate(EOS):
            key = f"d{dim}/{ename}"
            refpin.set_physics(gamma, b, R, dim)
            u1, u2, nor = inputs(dim, gamma, b, seed=100 + 10 * di + ei)
            data[f"{key}/u1"], data[f"{key}/u2"], data[f"{key}/nor"] = u1, u2, nor
            data[f"{key}/eos"] = refpin.eos(u1, dim)
            data[f"{key}/flux_full"] = refpin.flux(u1, dim)
            ok = (data[f"{key}/eos"][:, 4] > 0) & (refpin.eos(u2, dim)[:, 4] > 0)
            data[f"{key}/trrs"] = refpin.speeds(0, u1[ok], u2[ok], nor[ok])
            data[f"{key}/einfeldt"] = refpin.speeds(1, u1[ok], u2[ok], nor[ok])
            data[f"{key}/speeds_ok"] = ok
            for rs in range(4):
                f, sp = refpin.riemann(rs, u1, u2, nor)
                data[f"{key}/rs{rs}/flux"], data[f"{key}/rs{rs}/speed"] = f, sp
            s1, bnor, outer = bc_inputs(dim, gamma, b, seed=200 + 10 * di + ei)
            data[f"{key}/bc/s1"], data[f"{key}/bc/nor"] = s1, bnor
            data[f"{key}/bc/outer"] = outer
            prms = {0: None, 1: None, 2: outer, 3: outer, 4: None, 5: outer,
                    6: [1.3, 1.2], 7: [0.8, 1.2], 8: [0.7], 9: [1.3, 1.0]}
            for bc, prm in prms.items():
                data[f"{key}/bc{bc}"] = refpin.right_state(bc, s1, bnor, prm=prm)
                if prm is not None:
                    data[f"{key}/bc{bc}/prm"] = np.pad(np.ravel(np.asarray(prm, float)),
                                                       (0, dim + 2 - np.size(prm)))
            # characteristic outlet: state2 on entry = the interior state (a
            # stated seed; the reference reads whatever the previous point left)
            data[f"{key}/bc10"] = refpin.right_state(10, s1, bnor, prm=outer, s2_in=s1)
            # ... and chained: each point starts from the previous point's ghost
            chain = np.zeros_like(s1)
            prev = s1[:1]
            for i in range(s1.shape[0]):
                prev = refpin.right_state(10, s1[i:i + 1], bnor[i:i + 1], prm=outer, s2_in=prev)
                chain[i] = prev[0]
            data[f"{key}/bc10_chain"] = chain
    np.savez_compressed(OUT, **data)
    print("wrote", OUT, len(data), "arrays", os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    main()
