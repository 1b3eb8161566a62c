"""The laminar viscous term on the GPU.

* FP64-exact path against the oracle's restatement, bit-for-bit, on a box
  with no-slip walls, inlet, outlet and symmetry faces, several RK2 steps.
* Decay of a periodic shear wave u = U0 sin(2 pi y / L) against the
  analytic rate exp(-nu k^2 t) (low Mach, compressible Navier-Stokes): the
  amplitude after t = 5 within 1% of exact, FP64 and FP32.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _both(m):
    from mstcfd import Mesh
    from oracle import pyoracle as po
    sh = m.get("c1_shift")
    return (Mesh.from_arrays(m["node_xy"], m["face_nodes"], m["face_cells"], m["zones"],
                             m["n_cells"], c1_shift=sh),
            po.mesh_from_arrays(m["node_xy"], m["face_nodes"], m["face_cells"], m["zones"],
                                m["n_cells"], c1_shift=sh))


@pytest.mark.parametrize("flux", [0, 1], ids=["ausm", "roe"])
@pytest.mark.parametrize("limiter", [0, 2])
def test_exact_viscous_matches_oracle(flux, limiter):
    from mstcfd import Solver
    from mstcfd import meshgen as mg
    from oracle import pyoracle as po
    m = mg.tri_box(30, 16, 4.0, 2.0, jitter=0.2, seed=17)
    mesh, om = _both(m)
    q0 = mg.smooth_state(om.cell_ctr)
    kw = dict(flux=flux, order=2, limiter=limiter, reference_quirks=0, time_scheme=1,
              dt_mode=1, cfl=0.4, viscous=1, mu=0.02, lambda_=-2.0 / 3.0 * 0.02,
              kappa=0.03, cv=2.5)
    s = Solver(mesh, **kw)
    s.set_state(q0)
    s.step(3)
    prm = po.params_ext(flux, 2, limiter=limiter, quirks=0, rk2=1, dt_mode=1, cfl=0.4,
                        viscous=1, mu=0.02, lam=-2.0 / 3.0 * 0.02, kappa=0.03, cv=2.5)
    q, _ = po.step_ext(om, prm, q0, 3)
    assert np.array_equal(s.state(), q)


@pytest.mark.parametrize("prec", [1, 2], ids=["fp64", "fp32"])
def test_shear_wave_decay(prec):
    from mstcfd import Solver
    from mstcfd import meshgen as mg
    L, U0, mu = 10.0, 0.01, 0.05
    m = mg.periodic_delaunay(64, L, seed=3)
    mesh, om = _both(m)
    y = om.cell_ctr[:, 1]
    k = 2 * np.pi / L
    rho = np.ones(len(y))
    q0 = mg.primitive_to_q(rho, U0 * np.sin(k * y), 0 * y, np.ones(len(y)))
    s = Solver(mesh, flux=0, order=2, limiter=0, reference_quirks=0, time_scheme=1,
               dt_mode=1, cfl=0.5, viscous=1, mu=mu, lambda_=-2.0 / 3.0 * mu, kappa=0.0,
               cv=2.5, precision=prec)
    s.set_state(q0)
    t_end = 5.0
    while s.time() < t_end - 1e-12:
        s.step(50, t_end=t_end)
    q = s.state()
    u = q[:, 1] / q[:, 0]
    amp = 2 * np.sum(u * np.sin(k * y) * om.cell_vol) / np.sum(om.cell_vol)
    exact = U0 * np.exp(-mu * k * k * t_end)
    assert abs(amp - exact) < 0.01 * exact, (amp, exact)
