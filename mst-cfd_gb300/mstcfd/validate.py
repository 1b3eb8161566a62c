"""Accuracy statements of the benchmark configurations, run on the GPU.

  python -m mstcfd.validate vortex [--n 1000] [--periods 10] [--fp64-periods 10]

Isentropic vortex (strength 5, Mach 0.5) on the periodic jittered Delaunay
mesh, AUSM+ + van Leer, RK2 at CFL 0.5: the FP32 path advanced --periods
periods and the FP64 path --fp64-periods (default the same), with the L2
and L-infinity density errors of the FP32 path against the FP64 path (at
the FP64 path's end) and of both against the analytic solution (the vortex
convected back to its start).  One JSON line.

  python -m mstcfd.validate sod

Sod tube, 1000x4 quads, Roe + minmod, RK2 at CFL 0.5 to t = 0.2: the FP64
and FP32 paths against the exact Riemann solution (L1, L2, L-infinity of
density).

  python -m mstcfd.validate tgv [--tgv-n 128] [--t-end 10]

3D Taylor-Green vortex (Ma 0.1, Re 1600) on the periodic tetrahedral mesh,
FP32 path: kinetic-energy history and dissipation rate to t* = t-end
convective times.
"""
import argparse
import json
import sys
import time

import numpy as np


def _errors(a, b):
    d = a - b
    return {"l2": float(np.sqrt(np.mean(d * d))), "linf": float(np.abs(d).max())}


def vortex(n=1000, periods=10.0, fp64_periods=None, cfl=0.5):
    """FP32 path to `periods`, FP64 path to `fp64_periods` (default the
    same); errors against the analytic solution at each path's end, and
    FP32 against FP64 at the FP64 path's end (the FP32 state is kept
    there on its way)."""
    from . import Mesh, Solver
    from . import meshgen as mg
    m = mg.periodic_delaunay(n, 10.0, jitter=0.25, seed=20261203)
    mesh = Mesh.from_arrays(m["node_xy"], m["face_nodes"], m["face_cells"], m["zones"],
                            m["n_cells"], c1_shift=m["c1_shift"])
    xy = m["cell_centroid"]
    q0 = mg.isentropic_vortex(xy)
    period = 10.0 / (0.5 * np.sqrt(1.4))
    fp64_periods = periods if fp64_periods is None else fp64_periods
    out = {"workload": f"isentropic vortex, {m['n_cells']} triangles (lattice {n}x{n}), "
                       f"AUSM+ + van Leer, RK2, CFL {cfl}",
           "periods": {"fp32": periods, "fp64": fp64_periods}}
    snaps = {}

    def advance(s, t_end):
        steps = 0
        while s.time() < t_end - 1e-12:
            s.step(500, t_end=t_end)
            steps += 500
        return steps

    for prec, label, nper in ((2, "fp32", periods), (1, "fp64", fp64_periods)):
        s = Solver(mesh, flux=0, order=2, limiter=2, reference_quirks=0, time_scheme=1,
                   dt_mode=1, cfl=cfl, precision=prec)
        s.set_state(q0)
        t0 = time.perf_counter()
        ends = sorted({fp64_periods, nper}) if label == "fp32" else [nper]
        for e in ends:
            if e > nper:
                break
            advance(s, e * period)
            snaps[(label, e)] = s.state()
        out[label] = {"wall_s": round(time.perf_counter() - t0, 1), "time": s.time()}
        s.close()
    # after whole periods the vortex is back at its start
    for label, nper in (("fp32", periods), ("fp64", fp64_periods)):
        out[label]["vs_analytic"] = _errors(snaps[(label, nper)][:, 0], q0[:, 0])
    if ("fp32", fp64_periods) in snaps:
        out["fp32_vs_fp64"] = {"at_periods": fp64_periods,
                               **_errors(snaps[("fp32", fp64_periods)][:, 0],
                                         snaps[("fp64", fp64_periods)][:, 0])}
        out["fp32_vs_analytic_at_fp64_end"] = _errors(snaps[("fp32", fp64_periods)][:, 0],
                                                      q0[:, 0])
    return out


def sod():
    from . import Mesh, Solver
    from . import meshgen as mg
    from .analytic import riemann_sample
    m = mg.sod_strip(1000, 4, ends=mg.OUTLET)
    mesh = Mesh.from_arrays(m["node_xy"], m["face_nodes"], m["face_cells"], m["zones"],
                            m["n_cells"])
    x = mesh.arrays()["cell_ctr"][:, 0]
    rho_e, _, _ = riemann_sample(x, 0.2, 0.5, (1.0, 0.0, 1.0), (0.125, 0.0, 0.1))
    out = {"workload": "Sod tube, 1000x4 quads, Roe + minmod, RK2, CFL 0.5, t = 0.2"}
    for prec, label in ((1, "fp64"), (2, "fp32")):
        s = Solver(mesh, flux=1, order=2, limiter=1, reference_quirks=0, time_scheme=1,
                   dt_mode=1, cfl=0.5, precision=prec)
        s.set_state(mg.sod_state(mesh.arrays()["cell_ctr"]))
        while s.time() < 0.2 - 1e-15:
            s.step(100, t_end=0.2)
        rho = s.state()[:, 0]
        e = _errors(rho, rho_e)
        e["l1"] = float(np.mean(np.abs(rho - rho_e)))
        out[label] = e
        s.close()
    return out


def tgv(n=128, t_end=10.0, samples=20, precision=2):
    """Kinetic-energy history of the 3D Taylor-Green vortex (Ma 0.1,
    Re 1600) on the n^3 x 6 periodic tetrahedral mesh, in convective units
    (L = 1 per radian, V0 = Ma a = 0.1, t* = t V0 / L): E* = sum 1/2
    |rho u|^2 / rho V / (sum V rho0 V0^2) and the dissipation rate
    -dE*/dt* between samples.  For the initial field the laminar rate is
    (3/4) / Re = 4.69e-4 (nu <|grad u|^2> with <|grad u|^2> = 3 V0^2 / 4);
    the rest is the scheme's own dissipation."""
    from . import meshgen as mg
    from .mesh3d import Mesh3D
    from .solver3d import Solver3D
    m = mg.tet_grid(n, jitter=0.15, seed=20261205)
    q0 = mg.taylor_green(m["cell_centroid"], mach=0.1)
    mu = 0.1 / 1600.0
    cv = 1.0 / (1.4 * 0.4)
    s = Solver3D(Mesh3D.from_dict(m), precision=precision, order=2, limiter=3, viscous=1,
                 mu=mu, lambda_=-2.0 / 3.0 * mu, kappa=mu * 1.4 * cv / 0.71, cv=cv, cfl=0.5)
    s.set_state(q0)
    norm = 0.1 ** 2
    t_unit = 1.0 / 0.1  # L / V0
    ke, vol = s.kinetic_energy()
    hist = [(0.0, ke / vol / norm)]
    t0 = time.perf_counter()
    steps = 0
    t = s.step(10)
    dt_est = t / 10
    steps += 10
    for i in range(1, samples + 1):
        te = t_end * t_unit * i / samples
        while t < te - 1e-12:
            # steps of zero length past te are wasted: size the call
            n_call = max(1, int((te - t) / dt_est) + 2)
            t = s.step(n_call, t_end=te)
            steps += n_call
        ke, vol = s.kinetic_energy()
        hist.append((t / t_unit, ke / vol / norm))
    wall = time.perf_counter() - t0
    s.close()
    rate = [(0.5 * (a[0] + b[0]), -(b[1] - a[1]) / (b[0] - a[0])) for a, b in zip(hist, hist[1:])]
    return {"workload": f"Taylor-Green vortex, Ma 0.1, Re 1600, {n}^3 x 6 tetrahedra "
                        f"({m['n_cells']} cells), Roe + van Albada + viscous, RK2, CFL 0.5",
            "precision": {0: "fp64 exact", 1: "fp64", 2: "fp32"}[precision],
            "wall_s": round(wall, 1), "steps_upper_bound": steps,
            "time_unit": "t* = t V0 / L", "laminar_initial_rate": 0.75 / 1600.0,
            "kinetic_energy": [[round(t, 4), round(k, 6)] for t, k in hist],
            "dissipation_rate": [[round(t, 4), round(r, 6)] for t, r in rate],
            "peak_dissipation": max(rate, key=lambda x: x[1])}


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("case", choices=["vortex", "sod", "tgv"])
    ap.add_argument("--tgv-n", type=int, default=128)
    ap.add_argument("--t-end", type=float, default=10.0)
    ap.add_argument("--n", type=int, default=1000)
    ap.add_argument("--periods", type=float, default=10.0)
    ap.add_argument("--fp64-periods", type=float, default=None)
    a = ap.parse_args(argv)
    if a.case == "vortex":
        print(json.dumps(vortex(a.n, a.periods, a.fp64_periods)))
    elif a.case == "tgv":
        print(json.dumps(tgv(a.tgv_n, a.t_end)))
    else:
        print(json.dumps(sod()))


if __name__ == "__main__":
    sys.exit(main())
