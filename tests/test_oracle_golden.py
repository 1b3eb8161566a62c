"""The C oracle against the committed golden fixtures (made by the reference
itself, tests/golden/make_golden.py).  Runs on every machine."""
import os

import numpy as np
import pytest

from conftest import golden_cases, golden_msh, load_golden
from oracle import pyoracle as po

CASES = golden_cases()
IDS = [os.path.basename(c)[:-4] for c in CASES]


def _eq(a, b):
    return np.array_equal(np.asarray(a), np.asarray(b), equal_nan=True)


def test_fixtures_present():
    assert len(CASES) >= 3


@pytest.mark.parametrize("case", CASES, ids=IDS)
def test_geometry(case, tmp_path):
    g = load_golden(case)
    m = po.read_msh(golden_msh(g, tmp_path))
    for mine, k in [("cell_vol", "cell_volume"), ("cell_ctr", "cell_center"),
                    ("face_eta0", "face_eta0"), ("face_flag", "face_flag"),
                    ("face_dac", "face_dac"), ("cell_dof", "cell_dof"),
                    ("cell_faces", "cell_faces"), ("cell_nb", "cell_nbcells"),
                    ("bond1", "bond1"), ("bond2", "bond2"), ("inner", "inner")]:
        assert _eq(getattr(m, mine), g["geo_" + k]), mine


@pytest.mark.parametrize("case", CASES, ids=IDS)
@pytest.mark.parametrize("flux", ["ausm", "roe"])
@pytest.mark.parametrize("order", [1, 2])
def test_solve(case, flux, order, tmp_path):
    g = load_golden(case)
    m = po.read_msh(golden_msh(g, tmp_path))
    if order == 2:
        z = m.zone.copy()
        z[z[:, 3] == 5, 3] = 3
        m = po.mesh_from_arrays(m.node_xy, m.face_nodes, m.face_cells, z, m.n_cells)
    fl = po.ROE if flux == "roe" else po.AUSM
    q0 = g[f"q0_o{order}"]
    prm = po.params(fl, order)
    grad = po.gradient(m, q0)[1] if order == 2 else None
    F = po.face_flux(m, prm, q0, grad)
    qn, R = po.solve(m, prm, q0, float(g["dt"]))
    v = f"{flux}_o{order}"
    assert _eq(F, g[v + "_flux"])
    assert _eq(R, g[v + "_resid"])
    assert _eq(qn, g[v + "_qnew"])


@pytest.mark.parametrize("case", CASES, ids=IDS)
@pytest.mark.parametrize("flux", ["ausm", "roe"])
def test_time_loop(case, flux, tmp_path):
    g = load_golden(case)
    m = po.read_msh(golden_msh(g, tmp_path))
    fl = po.ROE if flux == "roe" else po.AUSM
    q = g[flux + "_steps_q0"].copy()
    rows = []
    for _ in range(len(g[flux + "_steps_log"])):
        qn, _ = po.solve(m, po.params(fl, 1), q, 1.0 / 4e3)
        rows.append(po.linf_change(q, qn))
        q = qn
    assert _eq(q, g[flux + "_steps_q"])
    assert np.allclose(rows, g[flux + "_steps_log"], rtol=0, atol=6e-16, equal_nan=True)


def _shipped():
    from conftest import GOLDEN
    p = os.path.join(GOLDEN, "shipped.npz")
    return load_golden(p) if os.path.exists(p) else None


SHIPPED = _shipped()
SHIPPED_NAMES = [str(x) for x in SHIPPED["meshes"]] if SHIPPED is not None else []


def _shipped_oracle_mesh(name, tmp_path, order):
    p = os.path.join(str(tmp_path), name + ".msh")
    with open(p, "wb") as f:
        f.write(bytes(SHIPPED[name + "_msh"]))
    m = po.read_msh(p)
    if order == 2:
        z = m.zone.copy()
        z[z[:, 3] == 5, 3] = 3
        m = po.mesh_from_arrays(m.node_xy, m.face_nodes, m.face_cells, z, m.n_cells)
    return m


@pytest.mark.parametrize("name", SHIPPED_NAMES)
@pytest.mark.parametrize("flux", ["ausm", "roe"])
@pytest.mark.parametrize("order", [1, 2])
def test_solve_on_shipped_meshes(name, flux, order, tmp_path):
    """The oracle on two of the reference's own Fluent meshes against the
    reference's outputs (digests of residuals and new states)."""
    from golden.make_golden import digest, gentle_state
    from mstcfd import meshgen as mg
    m = _shipped_oracle_mesh(name, tmp_path, order)
    q0 = mg.random_state(m.n_cells, seed=11) if order == 1 else gentle_state(m.n_cells, 12)
    assert digest(q0) == str(SHIPPED[f"{name}_q0_o{order}_sha"])
    qn, R = po.solve(m, po.params(po.ROE if flux == "roe" else po.AUSM, order), q0,
                     float(SHIPPED["dt"]))
    v = f"{name}_{flux}_o{order}"
    assert digest(R) == str(SHIPPED[v + "_resid_sha"])
    assert digest(qn) == str(SHIPPED[v + "_qnew_sha"])


@pytest.mark.parametrize("name", SHIPPED_NAMES)
@pytest.mark.parametrize("flux", ["ausm", "roe"])
def test_time_loop_on_shipped_meshes(name, flux, tmp_path):
    from golden.make_golden import digest
    m = _shipped_oracle_mesh(name, tmp_path, 1)
    fl = po.ROE if flux == "roe" else po.AUSM
    q = SHIPPED[f"{name}_{flux}_steps_q0"].copy()
    rows = []
    for _ in range(len(SHIPPED[f"{name}_{flux}_steps_log"])):
        qn, _ = po.solve(m, po.params(fl, 1), q, 1.0 / 4e3)
        rows.append(po.linf_change(q, qn))
        q = qn
    assert digest(q) == str(SHIPPED[f"{name}_{flux}_steps_q_sha"])
    assert np.allclose(rows, SHIPPED[f"{name}_{flux}_steps_log"], rtol=0, atol=6e-16,
                       equal_nan=True)
