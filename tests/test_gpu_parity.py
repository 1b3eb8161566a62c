"""GPU parity through the C ABI.

* FP64_EXACT (no FMA, reference operation order) against arrays the
  reference itself produced (golden fixtures): face flux matrices, per-cell
  residuals and updated states bit-for-bit, for AUSM+ and Roe at 1st and
  2nd order, on meshes with both orientation branches of the reference's
  left/right flags and every boundary type it handles; and the reference's
  own time loop (state and L-infinity rows) over five steps.
* The same against the C oracle on fresh random meshes (multi-tile,
  renumbered).
* FP64 (FMA) and FP32-flux/FP64-accumulate against FP64_EXACT within the
  tolerances written below.
"""
import os

import numpy as np
import pytest

from conftest import golden_cases, golden_msh, load_golden

pytestmark = pytest.mark.gpu

CASES = golden_cases()
IDS = [os.path.basename(c)[:-4] for c in CASES]


def _eq(a, b):
    return np.array_equal(np.asarray(a), np.asarray(b), equal_nan=True)


def _mesh_for(g, tmp_path, order):
    from mstcfd import Mesh
    from oracle import pyoracle as po
    path = golden_msh(g, tmp_path)
    if order == 1:
        return Mesh.read_msh(path)
    om = po.read_msh(path)
    z = om.zone.copy()
    z[z[:, 3] == 5, 3] = 3  # outlets as walls for 2nd order (see fixtures)
    return Mesh.from_arrays(om.node_xy, om.face_nodes, om.face_cells, z, om.n_cells)


@pytest.mark.parametrize("case", CASES, ids=IDS)
@pytest.mark.parametrize("flux", ["ausm", "roe"])
@pytest.mark.parametrize("order", [1, 2])
def test_exact_solve_matches_reference(case, flux, order, tmp_path):
    from mstcfd import FLUX_AUSM, FLUX_ROE, Solver
    g = load_golden(case)
    mesh = _mesh_for(g, tmp_path, order)
    s = Solver(mesh, flux=FLUX_ROE if flux == "roe" else FLUX_AUSM, order=order,
               dt=float(g["dt"]))
    s.set_state(g[f"q0_o{order}"])
    s.solve()
    v = f"{flux}_o{order}"
    assert _eq(s.residual(), g[v + "_resid"])
    assert _eq(s.new_state(), g[v + "_qnew"])
    assert _eq(s.face_flux(), g[v + "_flux"])


@pytest.mark.parametrize("case", CASES, ids=IDS)
@pytest.mark.parametrize("flux", ["ausm", "roe"])
def test_exact_time_loop_matches_reference(case, flux, tmp_path):
    from mstcfd import FLUX_AUSM, FLUX_ROE, Mesh, Solver
    g = load_golden(case)
    mesh = Mesh.read_msh(golden_msh(g, tmp_path))
    s = Solver(mesh, flux=FLUX_ROE if flux == "roe" else FLUX_AUSM)
    s.set_state(g[flux + "_steps_q0"])
    rows = []
    for _ in range(len(g[flux + "_steps_log"])):
        rows.append(s.step(1)["linf_change"])
    assert _eq(s.state(), g[flux + "_steps_q"])
    assert np.allclose(rows, g[flux + "_steps_log"], rtol=0, atol=6e-16, equal_nan=True)


def test_rhosolver_surface(tmp_path):
    """The RhoSolver mirror: setDT / solve / getNewValue / updateNewToOld."""
    from mstcfd import Mesh, RhoSolver
    g = load_golden(CASES[0])
    mesh = Mesh.read_msh(golden_msh(g, tmp_path))
    q = g["q0_o1"].copy()
    rs = RhoSolver(mesh, q)
    rs.setDT(float(g["dt"]))
    rs.solve()
    assert _eq(rs.getNewValue(), g["ausm_o1_qnew"])
    assert _eq(rs.getOldValue(), g["q0_o1"])
    rs.updateNewToOld()
    assert _eq(rs.getOldValue(), g["ausm_o1_qnew"])


@pytest.mark.parametrize("flux", [0, 1], ids=["ausm", "roe"])
@pytest.mark.parametrize("order", [1, 2])
@pytest.mark.parametrize("orient", ["into_c0", "random"])
def test_exact_matches_oracle_fresh_mesh(flux, order, orient):
    from mstcfd import Mesh, Solver
    from mstcfd import meshgen as mg
    from oracle import pyoracle as po
    m = mg.tri_box(48, 24, 4.0, 2.0, jitter=0.25, seed=21 + order)
    if orient == "random":
        m = mg.reorient(m, "random", seed=3)
    if order == 2:
        m = mg.with_zone_types(m, mg.OUTLET, mg.WALL)
    om = po.mesh_from_arrays(m["node_xy"], m["face_nodes"], m["face_cells"], m["zones"], m["n_cells"])
    q0 = mg.random_state(m["n_cells"], seed=5) if order == 1 else mg.smooth_state(om.cell_ctr)
    qn, R = po.solve(om, po.params(flux, order), q0, 2e-4)
    mesh = Mesh.from_arrays(m["node_xy"], m["face_nodes"], m["face_cells"], m["zones"], m["n_cells"])
    assert mesh.info.n_tiles > 8
    s = Solver(mesh, flux=flux, order=order, dt=2e-4)
    s.set_state(q0)
    s.solve()
    assert _eq(s.residual(), R)
    assert _eq(s.new_state(), qn)


def _scaled_err(a, b):
    """max over cells/components of |a-b| / max|b| per component."""
    scale = np.nanmax(np.abs(b), axis=0)
    scale[scale == 0] = 1
    return np.nanmax(np.abs(a - b) / scale)


@pytest.mark.parametrize("flux", [0, 1], ids=["ausm", "roe"])
@pytest.mark.parametrize("order", [1, 2])
def test_fast_precisions_against_exact(flux, order):
    from mstcfd import PREC_FP32, PREC_FP64, Mesh, Solver
    from mstcfd import meshgen as mg
    m = mg.tri_box(40, 20, 4.0, 2.0, jitter=0.2, seed=8)
    if order == 2:
        m = mg.with_zone_types(m, mg.OUTLET, mg.WALL)
    mesh = Mesh.from_arrays(m["node_xy"], m["face_nodes"], m["face_cells"], m["zones"], m["n_cells"])
    xy = mesh.arrays()["cell_ctr"]
    q0 = mg.smooth_state(xy)
    out = {}
    for prec in (0, PREC_FP64, PREC_FP32):
        s = Solver(mesh, flux=flux, order=order, precision=prec, dt=1e-4)
        s.set_state(q0)
        s.solve()
        out[prec] = s.residual()
    # FP64 with FMA: residuals within 1e-12 of the exact path (scaled by the
    # largest residual of each component)
    assert _scaled_err(out[PREC_FP64], out[0]) < 1e-12
    # FP32 reconstruction/flux, FP64 accumulation: within 2e-5
    assert _scaled_err(out[PREC_FP32], out[0]) < 2e-5


def test_deterministic_repeat():
    from mstcfd import PREC_FP32, Mesh, Solver
    from mstcfd import meshgen as mg
    m = mg.tri_box(40, 20, seed=12)
    mesh = Mesh.from_arrays(m["node_xy"], m["face_nodes"], m["face_cells"], m["zones"], m["n_cells"])
    q0 = mg.smooth_state(mesh.arrays()["cell_ctr"])
    res = []
    for _ in range(2):
        s = Solver(mesh, order=2, precision=PREC_FP32, dt=1e-4)
        s.set_state(q0)
        n = s.step(3)
        res.append((s.state(), n["l2_resid"]))
    assert res[0][0].tobytes() == res[1][0].tobytes()
    assert np.array_equal(res[0][1], res[1][1])


def _shipped():
    from conftest import GOLDEN
    path = os.path.join(GOLDEN, "shipped.npz")
    return load_golden(path) if os.path.exists(path) else None


SHIPPED = _shipped()
SHIPPED_NAMES = [str(x) for x in SHIPPED["meshes"]] if SHIPPED is not None else []


def _shipped_mesh(g, name, tmp_path, order):
    from mstcfd import Mesh
    from oracle import pyoracle as po
    p = os.path.join(str(tmp_path), name + ".msh")
    with open(p, "wb") as f:
        f.write(bytes(g[name + "_msh"]))
    if order == 1:
        return Mesh.read_msh(p)
    om = po.read_msh(p)
    z = om.zone.copy()
    z[z[:, 3] == 5, 3] = 3  # outlets as walls at 2nd order, as in the fixture
    return Mesh.from_arrays(om.node_xy, om.face_nodes, om.face_cells, z, om.n_cells)


@pytest.mark.parametrize("name", SHIPPED_NAMES)
@pytest.mark.parametrize("flux", ["ausm", "roe"])
@pytest.mark.parametrize("order", [1, 2])
def test_exact_solve_matches_reference_on_shipped_meshes(name, flux, order, tmp_path):
    """The reference's own Fluent meshes (triangles; quadrilaterals with
    NaN-volume cells): one FP64_EXACT solve through the C ABI, residuals and
    new states bit-identical to the reference's (SHA-256 digests, NaNs
    unified)."""
    from golden.make_golden import digest, gentle_state
    from mstcfd import FLUX_AUSM, FLUX_ROE, Solver
    from mstcfd import meshgen as mg
    g = SHIPPED
    mesh = _shipped_mesh(g, name, tmp_path, order)
    q0 = mg.random_state(mesh.n_cells, seed=11) if order == 1 else gentle_state(mesh.n_cells, 12)
    assert digest(q0) == str(g[f"{name}_q0_o{order}_sha"])
    s = Solver(mesh, flux=FLUX_ROE if flux == "roe" else FLUX_AUSM, order=order,
               dt=float(g["dt"]))
    s.set_state(q0)
    s.solve()
    v = f"{name}_{flux}_o{order}"
    r = s.residual()
    assert int(np.isnan(r).any(1).sum()) == int(g[v + "_resid_nan"])
    assert digest(r) == str(g[v + "_resid_sha"])
    assert digest(s.new_state()) == str(g[v + "_qnew_sha"])
    s.close()


@pytest.mark.parametrize("name", SHIPPED_NAMES)
@pytest.mark.parametrize("flux", ["ausm", "roe"])
def test_exact_time_loop_matches_reference_on_shipped_meshes(name, flux, tmp_path):
    from golden.make_golden import digest
    from mstcfd import FLUX_AUSM, FLUX_ROE, Solver
    g = SHIPPED
    mesh = _shipped_mesh(g, name, tmp_path, 1)
    s = Solver(mesh, flux=FLUX_ROE if flux == "roe" else FLUX_AUSM)
    s.set_state(g[f"{name}_{flux}_steps_q0"])
    rows = [s.step(1)["linf_change"] for _ in range(len(g[f"{name}_{flux}_steps_log"]))]
    assert digest(s.state()) == str(g[f"{name}_{flux}_steps_q_sha"])
    assert np.allclose(rows, g[f"{name}_{flux}_steps_log"], rtol=0, atol=6e-16, equal_nan=True)
    s.close()
