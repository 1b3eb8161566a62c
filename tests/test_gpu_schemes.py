"""GPU checks of the schemes the reference lacks (limiters, corrected
boundaries, periodic images, CFL steps, RK2), against the oracle's
restatement and against analytic solutions.

Tolerances: the FP64-exact path is compared bit-for-bit (states, time);
norms summed in a different order are compared to rtol 1e-12.  FP32 flux
paths are compared to the FP64 path with the error bounds written in each
test."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _eq(a, b):
    return np.array_equal(np.asarray(a), np.asarray(b), equal_nan=True)


def _box(order):
    from mstcfd import meshgen as mg
    m = mg.tri_box(36, 18, 4.0, 2.0, jitter=0.25, seed=31)
    return m


def _periodic(n=24):
    from mstcfd import meshgen as mg
    return mg.periodic_delaunay(n, 10.0, seed=4)


def _both(m):
    from mstcfd import Mesh
    from oracle import pyoracle as po
    sh = m.get("c1_shift")
    mesh = Mesh.from_arrays(m["node_xy"], m["face_nodes"], m["face_cells"], m["zones"],
                            m["n_cells"], c1_shift=sh)
    om = po.mesh_from_arrays(m["node_xy"], m["face_nodes"], m["face_cells"], m["zones"],
                             m["n_cells"], c1_shift=sh)
    return mesh, om


@pytest.mark.parametrize("flux", [0, 1], ids=["ausm", "roe"])
@pytest.mark.parametrize("limiter", [0, 1, 2, 3], ids=["none", "minmod", "vanleer", "vanalbada"])
@pytest.mark.parametrize("scheme", ["euler_fixed", "rk2_cfl", "rk2_local"])
@pytest.mark.parametrize("geom", ["box", "periodic"])
def test_exact_ext_matches_oracle(flux, limiter, scheme, geom):
    from mstcfd import Solver
    from mstcfd import meshgen as mg
    from oracle import pyoracle as po
    m = _box(2) if geom == "box" else _periodic()
    mesh, om = _both(m)
    q0 = mg.smooth_state(om.cell_ctr) if geom == "box" else mg.isentropic_vortex(om.cell_ctr)
    rk2 = scheme != "euler_fixed"
    dt_mode = {"euler_fixed": 0, "rk2_cfl": 1, "rk2_local": 2}[scheme]
    order = 2
    kw = dict(flux=flux, order=order, limiter=limiter, reference_quirks=0,
              time_scheme=int(rk2), dt_mode=dt_mode, dt=2e-3, cfl=0.4)
    s = Solver(mesh, **kw)
    s.set_state(q0)
    n = s.step(4)
    prm = po.params_ext(flux, order, limiter=limiter, quirks=0, rk2=int(rk2),
                        dt_mode=dt_mode, dt=2e-3, cfl=0.4)
    q, on = po.step_ext(om, prm, q0, 4)
    assert _eq(s.state(), q)
    assert n["time"] == on["time"]
    assert n["dt"] == on["dt"]
    assert np.array_equal(n["linf_change"], on["linf_change"])
    assert np.allclose(n["l2_resid"], on["l2_resid"], rtol=1e-12, atol=0)
    assert np.isclose(n["mass"], on["mass"], rtol=1e-13, atol=0)


def test_exact_quirk_free_first_order_matches_oracle():
    """Corrected left/right on a Fluent-oriented mesh (all faces backwards)."""
    from mstcfd import Solver
    from mstcfd import meshgen as mg
    from oracle import pyoracle as po
    m = mg.reorient(mg.tri_box(30, 15, seed=2), "fluent")
    mesh, om = _both(m)
    q0 = mg.random_state(m["n_cells"], seed=1)
    s = Solver(mesh, flux=1, reference_quirks=0, dt=1e-3)
    s.set_state(q0)
    s.solve()
    F = po.face_flux_ext(om, po.params_ext(1, 1, quirks=0), q0)
    R = po.gather(om, F)
    assert _eq(s.residual(), R)
    assert _eq(s.face_flux(), F)


def test_sod_profile_config1():
    """Config 1: Sod tube, 1000x4 quads, Roe + minmod, RK2 at CFL 0.5 to
    t = 0.2, slip walls, transmissive ends.  The FP64-exact GPU run
    reproduces the FP64 oracle to 1e-10 (here: bit-for-bit) and the density
    is within 1e-2 (L1) of the exact Riemann solution."""
    from mstcfd import Mesh, Solver
    from mstcfd import meshgen as mg
    from mstcfd.analytic import riemann_sample
    from oracle import pyoracle as po
    m = mg.sod_strip(1000, 4, ends=mg.OUTLET)
    mesh, om = _both(m)
    q0 = mg.sod_state(om.cell_ctr)
    kw = dict(flux=1, order=2, limiter=1, reference_quirks=0, time_scheme=1,
              dt_mode=1, cfl=0.5)
    s = Solver(mesh, **kw)
    s.set_state(q0)
    steps = 0
    while s.time() < 0.2 - 1e-15 and steps < 5000:
        s.step(50, t_end=0.2)
        steps += 50
    assert abs(s.time() - 0.2) < 1e-14
    q = s.state()
    prm = po.params_ext(1, 2, limiter=1, quirks=0, rk2=1, dt_mode=1, cfl=0.5)
    qo, on = po.step_ext(om, prm, q0, 100000, t_end=0.2)
    assert np.max(np.abs(q - qo)) <= 1e-10
    x = om.cell_ctr[:, 0]
    rho, u, p = riemann_sample(x, 0.2, 0.5, (1.0, 0.0, 1.0), (0.125, 0.0, 0.1))
    rho_n = q[:, 0]
    assert np.mean(np.abs(rho_n - rho)) < 1e-2
    # the profile is monotone up to small over/undershoots (TVD)
    assert rho_n.max() <= 1.0 + 1e-6 and rho_n.min() >= 0.125 - 1e-6


def test_vortex_fp32_vs_fp64_config2_small():
    """Config 2 in small: isentropic vortex on a periodic jittered Delaunay
    mesh, AUSM+ + van Leer, RK2 at CFL 0.5 over a tenth of a period.  FP32
    flux path within 1e-5 (L-inf, density) of the FP64 path; both within
    2e-2 (L2) of the analytic solution."""
    from mstcfd import Solver
    from mstcfd import meshgen as mg
    m = mg.periodic_delaunay(64, 10.0, seed=7)
    mesh, om = _both(m)
    q0 = mg.isentropic_vortex(om.cell_ctr)
    period = 10.0 / (0.5 * np.sqrt(1.4))
    t_end = 0.1 * period
    out = {}
    for prec in (1, 2):
        s = Solver(mesh, flux=0, order=2, limiter=2, reference_quirks=0, time_scheme=1,
                   dt_mode=1, cfl=0.5, precision=prec)
        s.set_state(q0)
        while s.time() < t_end - 1e-14:
            s.step(20, t_end=t_end)
        out[prec] = s.state()
    exact = mg.isentropic_vortex(om.cell_ctr, t=t_end)
    d = np.abs(out[2][:, 0] - out[1][:, 0]).max()
    assert d < 1e-5, d
    for prec in (1, 2):
        e = np.sqrt(np.mean((out[prec][:, 0] - exact[:, 0]) ** 2))
        assert e < 2e-2, (prec, e)


@pytest.mark.parametrize("prec", [0, 1, 2])
@pytest.mark.parametrize("flux", [0, 1], ids=["ausm", "roe"])
def test_free_stream_preserved(prec, flux):
    from mstcfd import Solver
    from mstcfd import meshgen as mg
    m = _periodic(20)
    mesh, om = _both(m)
    q0 = np.tile(mg.primitive_to_q(np.array(1.2), np.array(0.3), np.array(-0.2),
                                   np.array(0.9)), (m["n_cells"], 1))
    s = Solver(mesh, flux=flux, order=2, limiter=2, reference_quirks=0, precision=prec,
               time_scheme=1, dt_mode=1, cfl=0.5)
    s.set_state(q0)
    s.step(10)
    tol = 1e-12 if prec < 2 else 1e-5
    assert np.abs(s.state() - q0).max() < tol * np.abs(q0).max()


@pytest.mark.parametrize("prec", [1, 2])
def test_conservation_periodic(prec):
    from mstcfd import Solver
    from mstcfd import meshgen as mg
    m = _periodic(32)
    mesh, om = _both(m)
    q0 = mg.isentropic_vortex(om.cell_ctr)
    s = Solver(mesh, flux=0, order=2, limiter=2, reference_quirks=0, precision=prec,
               time_scheme=1, dt_mode=1, cfl=0.5)
    s.set_state(q0)
    s.step(20)
    V = om.cell_vol[:, None]
    before = (V * q0).sum(0)
    after = (V * s.state()).sum(0)
    assert np.all(np.abs(after - before) <= 1e-11 * np.abs(before).max())


@pytest.mark.parametrize("prec", [0, 1, 2])
def test_step_reports_divergence(prec):
    """A state that leaves the physical range (here one cell of negative
    pressure) makes mst_step return MST_EDIVERGED instead of stepping on
    silently with NaN; a physical state on the same context still steps."""
    from mstcfd import Solver, capi
    from mstcfd import meshgen as mg
    m = _periodic(16)
    mesh, om = _both(m)
    q0 = mg.isentropic_vortex(om.cell_ctr)
    s = Solver(mesh, flux=0, order=2, limiter=2, reference_quirks=0, precision=prec,
               time_scheme=1, dt_mode=1, cfl=0.5)
    s.set_state(q0)
    s.step(2)
    bad = q0.copy()
    bad[5, 3] = 0.1 * 0.5 * (bad[5, 1] ** 2 + bad[5, 2] ** 2) / bad[5, 0]  # E < kinetic: p < 0
    s.set_state(bad)
    with pytest.raises(capi.MstError) as e:
        s.step(3)
    assert e.value.status == capi.EDIVERGED
    s.set_state(q0)
    s.step(2)
    s.close()
