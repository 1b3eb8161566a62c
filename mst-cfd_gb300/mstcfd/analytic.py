"""Analytic solutions used to check the solver: the exact Riemann problem
for the 1D Euler equations (Toro, "Riemann Solvers and Numerical Methods
for Fluid Dynamics", ch. 4: Newton iteration on the star pressure) and the
isentropic vortex (in meshgen.isentropic_vortex)."""
import numpy as np

GAMMA = 1.4


def _f_k(p, rho, pk, ak, g):
    """Pressure function f_K(p) and its derivative for one side."""
    if p > pk:  # shock
        A = 2.0 / ((g + 1) * rho)
        B = (g - 1) / (g + 1) * pk
        s = np.sqrt(A / (p + B))
        return (p - pk) * s, s * (1 - 0.5 * (p - pk) / (B + p))
    # rarefaction
    r = p / pk
    f = 2 * ak / (g - 1) * (r ** ((g - 1) / (2 * g)) - 1)
    df = 1.0 / (rho * ak) * r ** (-(g + 1) / (2 * g))
    return f, df


def riemann_star(rl, ul, pl, rr, ur, pr, g=GAMMA):
    al, ar = np.sqrt(g * pl / rl), np.sqrt(g * pr / rr)
    p = max(1e-8, 0.5 * (pl + pr))
    for _ in range(100):
        fl, dfl = _f_k(p, rl, pl, al, g)
        fr, dfr = _f_k(p, rr, pr, ar, g)
        dp = (fl + fr + (ur - ul)) / (dfl + dfr)
        pn = max(1e-12, p - dp)
        if abs(pn - p) < 1e-14 * (pn + p):
            p = pn
            break
        p = pn
    fl, _ = _f_k(p, rl, pl, al, g)
    fr, _ = _f_k(p, rr, pr, ar, g)
    u = 0.5 * (ul + ur) + 0.5 * (fr - fl)
    return p, u


def riemann_sample(x, t, x0, left, right, g=GAMMA):
    """Exact solution (rho, u, p) at points x and time t > 0 for the
    Riemann problem with states left/right = (rho, u, p) split at x0."""
    rl, ul, pl = left
    rr, ur, pr = right
    ps, us = riemann_star(rl, ul, pl, rr, ur, pr, g)
    al, ar = np.sqrt(g * pl / rl), np.sqrt(g * pr / rr)
    s = (np.asarray(x, float) - x0) / t
    rho = np.empty_like(s)
    u = np.empty_like(s)
    p = np.empty_like(s)
    for i, si in enumerate(s):
        if si <= us:  # left of contact
            if ps > pl:  # left shock
                sl = ul - al * np.sqrt((g + 1) / (2 * g) * ps / pl + (g - 1) / (2 * g))
                if si <= sl:
                    rho[i], u[i], p[i] = rl, ul, pl
                else:
                    rho[i] = rl * (ps / pl + (g - 1) / (g + 1)) / ((g - 1) / (g + 1) * ps / pl + 1)
                    u[i], p[i] = us, ps
            else:  # left rarefaction
                shl = ul - al
                asl = al * (ps / pl) ** ((g - 1) / (2 * g))
                stl = us - asl
                if si <= shl:
                    rho[i], u[i], p[i] = rl, ul, pl
                elif si >= stl:
                    rho[i] = rl * (ps / pl) ** (1 / g)
                    u[i], p[i] = us, ps
                else:
                    c = 2 / (g + 1) + (g - 1) / ((g + 1) * al) * (ul - si)
                    rho[i] = rl * c ** (2 / (g - 1))
                    u[i] = 2 / (g + 1) * (al + (g - 1) / 2 * ul + si)
                    p[i] = pl * c ** (2 * g / (g - 1))
        else:  # right of contact
            if ps > pr:  # right shock
                sr = ur + ar * np.sqrt((g + 1) / (2 * g) * ps / pr + (g - 1) / (2 * g))
                if si >= sr:
                    rho[i], u[i], p[i] = rr, ur, pr
                else:
                    rho[i] = rr * (ps / pr + (g - 1) / (g + 1)) / ((g - 1) / (g + 1) * ps / pr + 1)
                    u[i], p[i] = us, ps
            else:  # right rarefaction
                shr = ur + ar
                asr = ar * (ps / pr) ** ((g - 1) / (2 * g))
                str_ = us + asr
                if si >= shr:
                    rho[i], u[i], p[i] = rr, ur, pr
                elif si <= str_:
                    rho[i] = rr * (ps / pr) ** (1 / g)
                    u[i], p[i] = us, ps
                else:
                    c = 2 / (g + 1) - (g - 1) / ((g + 1) * ar) * (ur - si)
                    rho[i] = rr * c ** (2 / (g - 1))
                    u[i] = 2 / (g + 1) * (-ar + (g - 1) / 2 * ur + si)
                    p[i] = pr * c ** (2 * g / (g - 1))
    return rho, u, p
