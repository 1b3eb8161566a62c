"""The reference's pressure-based SIMPLE solver (pSolver/SolverSIMPLE.cpp).

* oracle (C restatement) against the fixtures the reference's own
  SolverSIMPLE produced (tests/golden/simple.npz) and against the reference
  binary on the shipped meshes where it exists;
* GPU (one persistent cluster kernel per call, through the C ABI) against
  the same fixtures and against the oracle on larger generated meshes:
  cell and face (p, u, v, T), the Time loop's residual rows, the SIMPLE
  iteration rows and the Gauss-Seidel iteration counts, bit-for-bit, for
  every cluster size.
"""
import os
import tempfile

import numpy as np
import pytest

from conftest import GOLDEN, REF_MSH_DIR

from oracle import pyoracle as po

CASES = ["tri_iow", "tri_sym"]


def _bits(a):
    return np.ascontiguousarray(a, dtype=np.float64).view(np.int64)


def same(a, b):
    return a.shape == b.shape and np.array_equal(_bits(a), _bits(b))


def _fixture(name):
    with np.load(os.path.join(GOLDEN, "simple.npz")) as z:
        g = {k[len(name) + 1:]: z[k] for k in z.files if k.startswith(name + "_")}
    d = tempfile.mkdtemp(prefix="simple_fx_")
    path = os.path.join(d, name + ".msh")
    with open(path, "wb") as f:
        f.write(g["msh"].tobytes())
    g["path"] = path
    return g


def _starts(g):
    """(label, initial cell PUVT, initial face PUVT, steps)"""
    yield "init", g["init_puvt"], g["init_face"], int(g["steps"])
    yield "rand", g["rand_puvt"], g["init_face"], 2


# ---- oracle ----------------------------------------------------------------------
@pytest.mark.parametrize("name", CASES)
def test_oracle_matches_reference_fixture(name):
    g = _fixture(name)
    m = po.read_msh(g["path"])
    for lab, p0, f0, steps in _starts(g):
        pv, fc, rows, _, its = po.simple_step(m, p0, f0, steps)
        assert same(pv, g[f"{lab}_puvt_out"]), lab
        assert same(fc, g[f"{lab}_face_out"]), lab
        assert same(rows, g[f"{lab}_time_rows_out"]), lab
        assert np.array_equal(its.reshape(-1, 3), g[f"{lab}_gs_iters_out"]), lab


@pytest.mark.parametrize("name", CASES)
def test_fixture_initial_field_is_the_reference_one(name):
    """The reference's Time::initialization field equals q_to_puvt of the
    split initial state (so tests may form it without the reference)."""
    g = _fixture(name)
    m = po.read_msh(g["path"])
    q0 = np.array(po.reference_inlet())
    q = np.tile(q0, (m.n_cells, 1))
    right = m.cell_ctr[:, 0] > 0.5
    q[right, 0] *= 0.125
    q[right, 3] *= 0.1
    assert same(po.q_to_puvt(q), g["init_puvt"])
    assert same(np.tile(po.q_to_puvt(q0[None])[0], (m.n_faces, 1)), g["init_face"])


@pytest.mark.ref
@pytest.mark.parametrize("mesh", ["2d-shockwavepipe-2", "2d-stairW-1"])
def test_oracle_matches_reference_shipped(mesh, ref_available):
    if not ref_available:
        pytest.skip("reference sources not available")
    from oracle import refrun
    path = os.path.join(REF_MSH_DIR, mesh + ".msh")
    init = refrun.run_simple(path, steps=0)
    r = refrun.run_simple(path, steps=2)
    m = po.read_msh(path)
    pv, fc, rows, inner, its = po.simple_step(m, init["puvt"], init["face"], 2)
    assert same(pv, r["puvt"]) and same(fc, r["face"]) and same(rows, r["time_rows"])
    assert np.array_equal(its.reshape(-1, 3), r["gs_iters"])
    # the solver's own rows are logged with 6 significant digits
    ref_rows = r["inner_rows"]
    fin = np.isfinite(ref_rows)
    assert np.array_equal(fin, np.isfinite(inner.reshape(-1, 4)))
    assert np.allclose(inner.reshape(-1, 4)[fin], ref_rows[fin], rtol=1e-5, atol=0)


# ---- GPU -------------------------------------------------------------------------
def _gpu_solver(path, p0, f0, **kw):
    from mstcfd import Mesh
    from mstcfd.psolver import SimpleSolver
    mesh = Mesh.read_msh(path)
    return SimpleSolver(mesh, p0, f0, **kw), mesh


@pytest.mark.gpu
@pytest.mark.parametrize("name", CASES)
def test_gpu_matches_reference_fixture(name):
    g = _fixture(name)
    for lab, p0, f0, steps in _starts(g):
        s, _ = _gpu_solver(g["path"], p0, f0)
        rows = s.step(steps)
        pv, fc = s.state()
        _, its = s.rows()
        assert same(pv, g[f"{lab}_puvt_out"]), lab
        assert same(fc, g[f"{lab}_face_out"]), lab
        assert same(rows, g[f"{lab}_time_rows_out"]), lab
        assert np.array_equal(its.reshape(-1, 3), g[f"{lab}_gs_iters_out"]), lab


def _channel(nx, ny, seed):
    from mstcfd import meshgen as mg
    return mg.reorient(mg.tri_box(nx, ny, 2.0, 1.0, jitter=0.2, seed=seed, left=mg.INLET,
                                  right=mg.OUTLET, bottom=mg.WALL, top=mg.SYMMETRY),
                       "random", seed=seed + 1)


@pytest.mark.gpu
@pytest.mark.parametrize("cluster", [0, 1, 4])
def test_gpu_matches_oracle_generated(cluster):
    """A 2 x 60 x 40 triangle channel (inlet, outlet, wall, symmetry) from a
    random state: every cluster size gives the oracle's bits."""
    from mstcfd import meshgen as mg
    d = tempfile.mkdtemp(prefix="simple_gen_")
    path = os.path.join(d, "chan.msh")
    mg.write_msh(path, _channel(60, 40, 5))
    m = po.read_msh(path)
    rng = np.random.default_rng(3)
    n = m.n_cells
    p0 = np.stack([rng.uniform(0.5, 1.5, n), rng.uniform(-0.3, 0.3, n),
                   rng.uniform(-0.3, 0.3, n), rng.uniform(0.8, 1.2, n) / 286.32], 1)
    f0 = np.tile(po.q_to_puvt(np.array(po.reference_inlet())[None])[0], (m.n_faces, 1))
    pv, fc, rows, inner, its = po.simple_step(m, p0, f0, 3)
    s, _ = _gpu_solver(path, p0, f0, cluster=cluster)
    grows = s.step(3)
    gpv, gfc = s.state()
    ginner, gits = s.rows()
    assert same(gpv, pv) and same(gfc, fc) and same(grows, rows)
    assert same(ginner, inner) and np.array_equal(gits, its)
    if cluster:
        assert s.info().cluster == cluster


@pytest.mark.gpu
def test_gpu_steps_split_equal_one_call():
    """Two calls of 2 steps equal one call of 4 (old time level carried)."""
    g = _fixture("tri_iow")
    a, _ = _gpu_solver(g["path"], g["rand_puvt"], g["init_face"])
    b, _ = _gpu_solver(g["path"], g["rand_puvt"], g["init_face"])
    ra = np.concatenate([a.step(2), a.step(2)])
    rb = b.step(4)
    assert same(ra, rb)
    assert same(a.state()[0], b.state()[0])


@pytest.mark.gpu
def test_gpu_reference_call_surface():
    """PSolver: setDT / solve / getNewValue / getOldValue as the Time loop
    uses them (time/Time.cpp:57-78)."""
    from mstcfd import Mesh
    from mstcfd.psolver import PSolver
    g = _fixture("tri_sym")
    ps = PSolver(Mesh.read_msh(g["path"]), g["init_puvt"], g["init_face"])
    ps.setDT(1.0 / 4e3)
    for _ in range(int(g["steps"])):
        ps.solve()
        old, new = ps.getOldValue(), ps.getNewValue()
        ps.updateNewToOld()
    assert same(new, g["init_puvt_out"])
    assert not same(old, new)


def test_simple_rejects_periodic_mesh():
    pytest.importorskip("ctypes")
    from mstcfd import Mesh, capi, meshgen as mg
    from mstcfd.psolver import SimpleSolver
    m = mg.periodic_delaunay(60, 1.0)
    mesh = Mesh.from_arrays(m["node_xy"], m["face_nodes"], m["face_cells"], m["zones"],
                            m["n_cells"], c1_shift=m["c1_shift"])
    with pytest.raises(capi.MstError) as e:
        SimpleSolver(mesh)
    assert e.value.status == capi.EUNSUPPORTED


@pytest.mark.gpu
def test_gpu_batch_equals_single_cases():
    """Several cases in one launch (one cluster each) give each case's own
    single-launch bits."""
    from mstcfd.psolver import step_batch
    cases = []
    for name in CASES:
        g = _fixture(name)
        cases.append((g["path"], g["rand_puvt"], g["init_face"]))
    from mstcfd import meshgen as mg
    path = os.path.join(tempfile.mkdtemp(prefix="simple_b_"), "chan.msh")
    mg.write_msh(path, _channel(40, 30, 8))
    m = po.read_msh(path)
    f0 = np.tile(po.q_to_puvt(np.array(po.reference_inlet())[None])[0], (m.n_faces, 1))
    cases.append((path, None, f0))
    singles, batch = [], []
    for path, p0, f0 in cases:
        a, _ = _gpu_solver(path, p0, f0)
        b, _ = _gpu_solver(path, p0, f0)
        singles.append((a, a.step(3)))
        batch.append(b)
    rows = step_batch(batch, 3)
    for i, ((a, ra), b) in enumerate(zip(singles, batch)):
        assert same(rows[i], ra), i
        assert same(a.state()[0], b.state()[0]) and same(a.state()[1], b.state()[1]), i
        ia, ib = a.rows(), b.rows()
        assert same(ia[0], ib[0]) and np.array_equal(ia[1], ib[1]), i
