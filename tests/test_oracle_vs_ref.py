"""Pins the C oracle against the reference itself, compiled here from its
own sources (oracle/_ref).  Runs only where the reference checkout exists;
elsewhere the committed golden fixtures carry the same evidence."""
import os

import numpy as np
import pytest

from conftest import shipped_meshes
from oracle import pyoracle as po

pytestmark = pytest.mark.ref

GEOM = [("cell_vol", "cell_volume"), ("cell_ctr", "cell_center"),
        ("face_ctr", "face_center"), ("face_dir", "face_direct"),
        ("face_area", "face_area"), ("face_eta0", "face_eta0"),
        ("face_dac", "face_dac"), ("face_flag", "face_flag"),
        ("cell_dof", "cell_dof"), ("cell_eta0c", "cell_eta0c"),
        ("cell_ptr", "cell_ptr"), ("cell_faces", "cell_faces"),
        ("cell_nb", "cell_nbcells"), ("face_cells", "face_cells"),
        ("inner", "inner"), ("bond1", "bond1"), ("bond2", "bond2"),
        ("zone", "zones")]


def _eq(a, b):
    a, b = np.asarray(a), np.asarray(b)
    if a.shape != b.shape:
        return False
    if a.dtype.kind == "f":
        return np.array_equal(a, b, equal_nan=True)
    return np.array_equal(a, b)


def _rand_q(n, seed):
    r = np.random.default_rng(seed)
    rho, p = r.uniform(0.5, 1.5, n), r.uniform(0.5, 1.5, n)
    u, v = r.uniform(-2, 2, n), r.uniform(-2, 2, n)
    return np.stack([rho, rho * u, rho * v, p / 0.4 + 0.5 * rho * (u * u + v * v)], 1)


def _smooth_q(xy):
    x, y = xy[:, 0], xy[:, 1]
    rho = 1 + 0.2 * np.sin(3.1 * x) * np.cos(2.3 * y)
    u = 0.5 * np.cos(1.7 * x) * np.sin(2.9 * y)
    v = 0.5 * np.sin(2.2 * x) * np.cos(1.3 * y)
    p = 1 + 0.2 * np.cos(2.7 * x) * np.sin(1.9 * y)
    return np.stack([rho, rho * u, rho * v, p / 0.4 + 0.5 * rho * (u * u + v * v)], 1)


MESHES = shipped_meshes()


@pytest.mark.parametrize("path", MESHES, ids=[os.path.basename(m) for m in MESHES])
def test_reader_geometry_bit_exact(ref_available, path):
    from oracle import refrun
    m = po.read_msh(path)
    r = refrun.run(path, 0, 1)
    for mine, theirs in GEOM:
        assert _eq(getattr(m, mine), getattr(r, theirs)), mine


@pytest.mark.parametrize("path", MESHES, ids=[os.path.basename(m) for m in MESHES])
@pytest.mark.parametrize("flux", [po.AUSM, po.ROE], ids=["ausm", "roe"])
@pytest.mark.parametrize("order", [1, 2])
def test_solve_bit_exact(ref_available, path, flux, order):
    """One RhoSolver::solve(): per-cell residual and updated state."""
    from oracle import refrun
    m = po.read_msh(path)
    if order == 1:
        q0 = _rand_q(m.n_cells, 7)
    else:
        q0 = _smooth_q(m.cell_ctr)
        z = m.zone.copy()
        z[z[:, 3] == 5, 3] = 3
        m = po.mesh_from_arrays(m.node_xy, m.face_nodes, m.face_cells, z, m.n_cells)
    r = refrun.run(path, flux, order, q0=q0, dt=1e-3, remap5=(order == 2))
    qn, R = po.solve(m, po.params(flux, order), q0, 1e-3)
    assert _eq(R, r.resid)
    assert _eq(qn, r.qnew)
    if order == 2:
        faceq, _ = po.gradient(m, q0)
        assert _eq(faceq, r.faceq)


@pytest.mark.parametrize("path", MESHES[:3], ids=[os.path.basename(m) for m in MESHES[:3]])
@pytest.mark.parametrize("flux", [po.AUSM, po.ROE], ids=["ausm", "roe"])
def test_time_loop(ref_available, path, flux):
    """Time::goNextTimeStep: Sod start, DT = 1/STEP_TIME, L-inf residual."""
    from oracle import refrun
    r = refrun.run(path, flux, 1, time_steps=6)
    m = po.read_msh(path)
    q = r.q0.copy()
    rows = []
    for _ in range(6):
        qn, _ = po.solve(m, po.params(flux, 1), q, 1.0 / 4e3)
        rows.append(po.linf_change(q, qn))
        q = qn
    assert _eq(q, r.q_steps)
    log = r.time_log()
    # the log holds 15 fixed decimals
    assert np.allclose(np.array(rows), log, rtol=0, atol=6e-16, equal_nan=True)
