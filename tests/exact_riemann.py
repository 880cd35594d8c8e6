"""Exact solution of the 1D Riemann problem for a perfect gas (test
infrastructure).  Follows the standard textbook construction (Toro,
"Riemann Solvers and Numerical Methods for Fluid Dynamics", ch. 4): Newton
iteration on the pressure function for p*, then self-similar sampling."""
from __future__ import annotations

import numpy as np


def _fk(p, rho, pk, ck, g):
    if p > pk:
        A = 2.0 / ((g + 1.0) * rho)
        B = (g - 1.0) / (g + 1.0) * pk
        f = (p - pk) * np.sqrt(A / (p + B))
        df = np.sqrt(A / (B + p)) * (1.0 - 0.5 * (p - pk) / (B + p))
    else:
        f = 2.0 * ck / (g - 1.0) * ((p / pk) ** ((g - 1.0) / (2.0 * g)) - 1.0)
        df = 1.0 / (rho * ck) * (p / pk) ** (-(g + 1.0) / (2.0 * g))
    return f, df


def star_state(rl, ul, pl, rr, ur, pr, g=1.4):
    cl = np.sqrt(g * pl / rl)
    cr = np.sqrt(g * pr / rr)
    p = max(1e-8, 0.5 * (pl + pr) - 0.125 * (ur - ul) * (rl + rr) * (cl + cr))
    for _ in range(100):
        fl, dfl = _fk(p, rl, pl, cl, g)
        fr, dfr = _fk(p, rr, pr, cr, g)
        dp = (fl + fr + ur - ul) / (dfl + dfr)
        p = max(1e-10, p - dp)
        if abs(dp) < 1e-14 * p:
            break
    fl, _ = _fk(p, rl, pl, cl, g)
    fr, _ = _fk(p, rr, pr, cr, g)
    u = 0.5 * (ul + ur) + 0.5 * (fr - fl)
    return p, u


def sample(x, t, x0, left, right, g=1.4):
    """Primitive (rho, u, p) at positions x and time t."""
    rl, ul, pl = left
    rr, ur, pr = right
    ps, us = star_state(rl, ul, pl, rr, ur, pr, g)
    cl = np.sqrt(g * pl / rl)
    cr = np.sqrt(g * pr / rr)
    out = np.zeros((3, np.size(x)))
    for i, xi in enumerate(np.atleast_1d(x)):
        s = (xi - x0) / t
        if s <= us:
            if ps > pl:
                sl = ul - cl * np.sqrt((g + 1) / (2 * g) * ps / pl + (g - 1) / (2 * g))
                if s <= sl:
                    out[:, i] = (rl, ul, pl)
                else:
                    r = rl * (ps / pl + (g - 1) / (g + 1)) / ((g - 1) / (g + 1) * ps / pl + 1)
                    out[:, i] = (r, us, ps)
            else:
                shl = ul - cl
                csl = cl * (ps / pl) ** ((g - 1) / (2 * g))
                stl = us - csl
                if s <= shl:
                    out[:, i] = (rl, ul, pl)
                elif s > stl:
                    out[:, i] = (rl * (ps / pl) ** (1 / g), us, ps)
                else:
                    u = 2 / (g + 1) * (cl + (g - 1) / 2 * ul + s)
                    c = 2 / (g + 1) * (cl + (g - 1) / 2 * (ul - s))
                    r = rl * (c / cl) ** (2 / (g - 1))
                    out[:, i] = (r, u, pl * (c / cl) ** (2 * g / (g - 1)))
        else:
            if ps > pr:
                sr = ur + cr * np.sqrt((g + 1) / (2 * g) * ps / pr + (g - 1) / (2 * g))
                if s >= sr:
                    out[:, i] = (rr, ur, pr)
                else:
                    r = rr * (ps / pr + (g - 1) / (g + 1)) / ((g - 1) / (g + 1) * ps / pr + 1)
                    out[:, i] = (r, us, ps)
            else:
                shr = ur + cr
                csr = cr * (ps / pr) ** ((g - 1) / (2 * g))
                str_ = us + csr
                if s >= shr:
                    out[:, i] = (rr, ur, pr)
                elif s <= str_:
                    out[:, i] = (rr * (ps / pr) ** (1 / g), us, ps)
                else:
                    u = 2 / (g + 1) * (-cr + (g - 1) / 2 * ur + s)
                    c = 2 / (g + 1) * (cr - (g - 1) / 2 * (ur - s))
                    r = rr * (c / cr) ** (2 / (g - 1))
                    out[:, i] = (r, u, pr * (c / cr) ** (2 * g / (g - 1)))
    return out
