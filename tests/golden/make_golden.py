"""Generate the committed golden vectors (tests/golden/golden.npz).

The reference ships no tests or golden outputs and cannot be built here (MFEM
is absent), so these vectors come from the CPU oracle (oracle/refcpu) on
small deterministic cases.  They pin the oracle against regressions and are
the fixtures the GPU parity tests compare with.  Regenerate with

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle.refcpu import Oracle  # noqa: E402
from rkdg3d_gb300 import cases  # noqa: E402
from rkdg3d_gb300 import mesh as M  # noqa: E402
from rkdg3d_gb300.solver import (AVG_EINFELDT, AVG_TRRS, BC_SLIP, BC_SUPERSONIC_INLET,  # noqa: E402
                                 FUN_MICHALAK, FUN_VENKATAKRISHNAN, IND_BJ, LIM_MULTI, RS_HLL,
                                 RS_HLLC, RS_LLF, RS_RUSANOV, TABLEAU_REFERENCE_RK3)
from tests.helpers import periodic_case, random_state, walled_case  # noqa: E402


def golden_cases():
    """name -> (case, seed, dt).  Deterministic: meshes and states are rebuilt
    from these parameters by the tests."""
    out = {}
    c = cases.sod(nx=20, ny=2, rsolver=RS_HLLC, averaging=AVG_EINFELDT, function=FUN_MICHALAK,
                  tableau=TABLEAU_REFERENCE_RK3)
    out["sod_q1_hllc"] = (c, None, 2e-3)
    c = periodic_case(M.GEOM_SQUARE, 3, 2, RS_RUSANOV)
    out["quad_q2_rusanov_periodic"] = (c, 11, 1e-3)
    c = walled_case(M.GEOM_TRIANGLE, 4, 1, RS_HLL, AVG_TRRS, bc=BC_SLIP)
    c.limiter = (LIM_MULTI, IND_BJ, FUN_VENKATAKRISHNAN, 1, 0)
    out["tri_p1_hll_slip"] = (c, 12, 1e-3)
    c = periodic_case(M.GEOM_CUBE, 3, 1, RS_HLLC, AVG_TRRS)
    out["hex_q1_hllc_periodic"] = (c, 13, 1e-3)
    c = walled_case(M.GEOM_CUBE, 2, 2, RS_LLF, AVG_EINFELDT, covolume=0.01, bc=BC_SUPERSONIC_INLET)
    st = cases.supersonic_inlet_state(1.1, 0.3, -0.2, 0.1, 0.9, 1.4, 3)
    c.bcs = [(a, BC_SUPERSONIC_INLET, st) for a, _, _ in c.bcs]
    out["hex_q2_llf_covolume_inlet"] = (c, 14, 5e-4)
    return out


def initial_state(case, orc, seed):
    if seed is None:
        return cases.project(case, orc.node_coords())
    return random_state(orc.node_coords(), b=case.covolume, seed=seed, amp=0.2, vel=0.3)


def main():
    data = {}
    for name, (case, seed, dt) in golden_cases().items():
        orc = Oracle(case.mesh, case.order)
        cases.configure_oracle(case, orc)
        x = initial_state(case, orc, seed)
        y, mcs = orc.rhs(x)
        xl = orc.limit(x)
        xs, mcs_s = orc.step(x, dt)
        data[f"{name}/x"] = x
        data[f"{name}/rhs"] = y
        data[f"{name}/mcs"] = np.array([mcs])
        data[f"{name}/limited"] = xl
        data[f"{name}/step"] = xs
        data[f"{name}/step_mcs"] = np.array([mcs_s])
        data[f"{name}/means"] = orc.means(x)
    np.savez_compressed(os.path.join(HERE, "golden.npz"), **data)
    print("wrote", os.path.join(HERE, "golden.npz"), len(data), "arrays")


if __name__ == "__main__":
    main()
