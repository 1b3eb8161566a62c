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
