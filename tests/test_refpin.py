"""The oracle pinned to the reference's own arithmetic (no GPU).

tests/golden/refpin.npz holds inputs and outputs of the reference's
physics/physics.cpp, riemannsolvers/rs_*.cpp and bc/boundary_integrator_*.cpp,
compiled unmodified (oracle/refshim, ``make -C oracle ref``; script
tests/golden/make_refpin.py).  Where the reference tree is present the
fixture is re-derived from the compiled reference and must match bit for
bit; everywhere, the oracle's restatement must reproduce it.
"""
import os

import numpy as np
import pytest

from oracle import refpin
from oracle.refcpu import Oracle
from rkdg3d_gb300 import mesh as M
from tests.golden.make_refpin import EOS, bc_inputs, inputs

GOLD = os.path.join(os.path.dirname(__file__), "golden", "refpin.npz")
KEYS = [(dim, e) for dim in (2, 3) for e in EOS]
IDS = [f"d{d}-{e[0]}" for d, e in KEYS]


def _oracle(dim, gamma, b, R, rs=0, avg=0):
    mesh = M.hex_grid(3, 3, 3) if dim == 3 else M.quad_grid(3, 3, 0, 1, 0, 1, periodic=(True, True))
    o = Oracle(mesh, 1)
    o.set_physics(rs, avg, gamma, b, R)
    return o


def _close(a, b, tol):
    """Elementwise relative agreement, with an absolute floor at tol * max|b|."""
    a, b = np.asarray(a), np.asarray(b)
    scale = max(float(np.abs(b).max()), 1e-300)
    return np.all(np.abs(a - b) <= tol * np.maximum(np.abs(b), 1e-3 * scale))


@pytest.mark.parametrize("dim,eos", KEYS, ids=IDS)
def test_fixture_inputs_are_reproducible(dim, eos):
    g = np.load(GOLD)
    ei = EOS.index(eos)
    di = (2, 3).index(dim)
    u1, u2, nor = inputs(dim, eos[1], eos[2], seed=100 + 10 * di + ei)
    key = f"d{dim}/{eos[0]}"
    assert np.array_equal(u1, g[f"{key}/u1"]) and np.array_equal(u2, g[f"{key}/u2"])
    assert np.array_equal(nor, g[f"{key}/nor"])
    s1, bnor, outer = bc_inputs(dim, eos[1], eos[2], seed=200 + 10 * di + ei)
    assert np.array_equal(s1, g[f"{key}/bc/s1"]) and np.array_equal(bnor, g[f"{key}/bc/nor"])


@pytest.mark.skipif(not refpin.available(), reason="reference source tree absent")
@pytest.mark.parametrize("dim,eos", KEYS, ids=IDS)
def test_reference_library_reproduces_fixture(dim, eos):
    """The committed vectors are what the compiled reference computes."""
    g = np.load(GOLD)
    key = f"d{dim}/{eos[0]}"
    _, gamma, b, R = eos
    refpin.set_physics(gamma, b, R, dim)
    u1, u2, nor = g[f"{key}/u1"], g[f"{key}/u2"], g[f"{key}/nor"]
    assert np.array_equal(refpin.eos(u1, dim), g[f"{key}/eos"], equal_nan=True)
    for rs in range(4):
        f, sp = refpin.riemann(rs, u1, u2, nor)
        assert np.array_equal(f, g[f"{key}/rs{rs}/flux"], equal_nan=True)
        assert np.array_equal(sp, g[f"{key}/rs{rs}/speed"])
    s1, bnor = g[f"{key}/bc/s1"], g[f"{key}/bc/nor"]
    for bc in range(10):
        prm = g[f"{key}/bc{bc}/prm"] if f"{key}/bc{bc}/prm" in g else None
        assert np.array_equal(refpin.right_state(bc, s1, bnor, prm=prm), g[f"{key}/bc{bc}"])
    outer = g[f"{key}/bc/outer"]
    assert np.array_equal(refpin.right_state(10, s1, bnor, prm=outer, s2_in=s1), g[f"{key}/bc10"])


@pytest.mark.parametrize("dim,eos", KEYS, ids=IDS)
def test_oracle_eos_flux_and_speeds_match_reference(dim, eos):
    g = np.load(GOLD)
    key = f"d{dim}/{eos[0]}"
    _, gamma, b, R = eos
    o = _oracle(dim, gamma, b, R)
    u1, u2, nor = g[f"{key}/u1"], g[f"{key}/u2"], g[f"{key}/nor"]
    ref = g[f"{key}/eos"]
    got = o.pointwise(0, u1)
    assert np.array_equal(got[:, 3], ref[:, 4])           # StateIsPhysical
    phys = ref[:, 4] > 0
    assert np.array_equal(got[phys, :3], ref[phys, :3])   # p, c, max speed: bitwise
    neq = dim + 2
    F = o.pointwise(1, u1).reshape(-1, neq, dim)
    assert np.array_equal(F[phys], g[f"{key}/flux_full"][phys])
    ok = g[f"{key}/speeds_ok"]
    assert np.array_equal(o.pointwise(2, u1[ok], u2[ok], nor[ok]), g[f"{key}/trrs"])
    assert np.array_equal(o.pointwise(3, u1[ok], u2[ok], nor[ok]), g[f"{key}/einfeldt"])


@pytest.mark.parametrize("rs", [0, 1, 2, 3], ids=["rusanov", "llf", "hll", "hllc"])
@pytest.mark.parametrize("dim,eos", KEYS, ids=IDS)
def test_oracle_riemann_matches_reference(dim, eos, rs):
    """RiemannSolver*::Eval with TRRS speeds (the only averaging the
    reference's solvers call): fluxes and returned speeds, -1 on the same
    non-physical inputs."""
    g = np.load(GOLD)
    key = f"d{dim}/{eos[0]}"
    _, gamma, b, R = eos
    o = _oracle(dim, gamma, b, R, rs=rs)
    u1, u2, nor = g[f"{key}/u1"], g[f"{key}/u2"], g[f"{key}/nor"]
    f, sp = o.riemann(u1, u2, nor)
    ref_f, ref_sp = g[f"{key}/rs{rs}/flux"], g[f"{key}/rs{rs}/speed"]
    assert np.array_equal(sp == -1.0, ref_sp == -1.0)
    ok = ref_sp != -1.0
    assert (~ok).sum() >= 4
    assert np.array_equal(sp[ok], ref_sp[ok])
    assert np.array_equal(f[ok], ref_f[ok])


BC_NAMES = ["slip", "open", "constant", "supersonic_inlet", "wall", "subsonic_inlet",
            "subsonic_inlet_total_p", "subsonic_inlet_fixed_p", "fixed_p_outlet", "total_p_outlet",
            "char_outlet"]


@pytest.mark.parametrize("bc", range(11), ids=BC_NAMES)
@pytest.mark.parametrize("dim,eos", KEYS, ids=IDS)
def test_oracle_ghost_states_match_reference(dim, eos, bc):
    """computeRightState of every boundary condition of the factory.  The
    characteristic outlet reads its ghost vector before assigning it; the
    library and the oracle let it enter as the interior state, and the
    fixture called the reference's code with that entry value.  The
    total-pressure outlet reads the normal one past its end (nor[1..dim],
    boundary_integrator_open_total_pressure.cpp);
    the oracle forms m.n from the normal's own components, so it is compared
    where both give m.n the same sign (the only use of m.n)."""
    g = np.load(GOLD)
    key = f"d{dim}/{eos[0]}"
    _, gamma, b, R = eos
    o = _oracle(dim, gamma, b, R)
    prm = g[f"{key}/bc{bc}/prm"] if f"{key}/bc{bc}/prm" in g else None
    if bc == 10:
        prm = g[f"{key}/bc/outer"]
    o.set_bc(1, bc, prm)
    s1, nor, ref = g[f"{key}/bc/s1"], g[f"{key}/bc/nor"], g[f"{key}/bc{bc}"]
    keep = np.ones(len(s1), bool)
    if bc == 9:
        padded = np.concatenate([nor, np.zeros((len(nor), 1))], axis=1)
        ref_mn = (s1[:, 1:1 + dim] * padded[:, 1:1 + dim]).sum(1)
        own_mn = (s1[:, 1:1 + dim] * nor).sum(1)
        keep = (ref_mn > 0) == (own_mn > 0)
        assert keep.sum() >= 16
    got = np.array([o.right_state(1, s1[i], nor[i]) for i in range(len(s1))])
    assert np.array_equal(got[keep], ref[keep])
