"""Result writer and checkpoint files (work/Work.cpp:204-319, :432-514).

* oracle against the reference's own Work members (oracle/ref/harness_io.cpp):
  the Tecplot file byte-for-byte on generated meshes and on the shipped
  meshes (nodes that touch a face type the reference leaves unset, such as
  symmetry, are excluded there), the text checkpoint byte-for-byte and its
  read-back;
* oracle against the committed fixture tests/golden/writer.npz (the
  reference's bytes), so the GPU tests need no reference;
* GPU (through the C ABI): the reference-mode file byte-identical to the
  reference's, node averages bit-identical to the oracle in both weighting
  rules and on the FP32 path, the corrected-mode file a valid Tecplot zone,
  text checkpoints identical to the reference's, and the binary checkpoint
  restarting bit-for-bit, rejecting other meshes and corrupted files.
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN, shipped_meshes

IO_CASES = ["tri_iow", "quad_strip"]


def _golden():
    with np.load(os.path.join(GOLDEN, "writer.npz")) as z:
        return {k: z[k] for k in z.files}


def _msh(g, name, tmp_path):
    p = os.path.join(str(tmp_path), name + ".msh")
    with open(p, "wb") as f:
        f.write(bytes(g[name + "_msh"]))
    return p


# ---------------------------------------------------------------------------
# oracle
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("name", IO_CASES)
def test_oracle_matches_golden(name, tmp_path):
    from oracle import pyoracle as po
    g = _golden()
    om = po.read_msh(_msh(g, name, tmp_path))
    out = os.path.join(str(tmp_path), "o.plt")
    po.write_plt(om, g[name + "_q"], out, zone_t=7)
    assert open(out, "rb").read() == bytes(g[name + "_plt"])
    cell = os.path.join(str(tmp_path), "o.cell")
    po.write_cell_text(g[name + "_q"], cell)
    assert open(cell, "rb").read() == bytes(g[name + "_cell"])


def test_golden_readback_is_15_decimals():
    g = _golden()
    for name in IO_CASES:
        assert np.abs(g[name + "_readback"] - g[name + "_q"]).max() <= 5e-16 * 4


def _unset_nodes(om):
    """Nodes on a face whose type the reference's writer leaves unset."""
    bad = ~np.isin(om.face_type, [2, 3, 5, 10])
    return np.unique(om.face_nodes[bad].ravel())


@pytest.mark.ref
@pytest.mark.parametrize("path", shipped_meshes(), ids=os.path.basename)
def test_oracle_matches_reference_shipped(ref_available, path, tmp_path):
    from mstcfd import meshgen as mg
    from oracle import pyoracle as po
    from oracle import refrun
    om = po.read_msh(path)
    q = mg.random_state(om.n_cells, seed=3)
    plt, cell, back = refrun.run_io(path, q, zone_t=3, time_now=2)
    out = os.path.join(str(tmp_path), "o.plt")
    po.write_plt(om, q, out, zone_t=3)
    mine = open(out, "rb").read().split(b"\n")
    ref = plt.split(b"\n")
    assert len(mine) == len(ref)
    skip = set(int(n) + 3 for n in _unset_nodes(om))  # 3 header lines
    diff = [i for i, (a, b) in enumerate(zip(mine, ref)) if a != b and i not in skip]
    assert diff == []
    c = os.path.join(str(tmp_path), "o.cell")
    po.write_cell_text(q, c)
    assert open(c, "rb").read() == cell


@pytest.mark.ref
@pytest.mark.parametrize("seed", [1, 2])
def test_oracle_matches_reference_generated(ref_available, seed, tmp_path):
    from mstcfd import meshgen as mg
    from oracle import pyoracle as po
    from oracle import refrun
    m = mg.reorient(mg.tri_box(20, 11, 2.0, 1.0, jitter=0.25, seed=seed, left=mg.INLET,
                               right=mg.OUTLET, bottom=mg.WALL, top=mg.OUTLET),
                    "random", seed=seed)
    p = os.path.join(str(tmp_path), "g.msh")
    mg.write_msh(p, m)
    q = mg.random_state(int(m["n_cells"]), seed=seed)
    plt, cell, back = refrun.run_io(p, q, zone_t=seed, time_now=9)
    om = po.read_msh(p)
    out = os.path.join(str(tmp_path), "o.plt")
    po.write_plt(om, q, out, zone_t=seed)
    assert open(out, "rb").read() == plt


def _shoelace(xy):
    x, y = xy[..., 0], xy[..., 1]
    return 0.5 * np.abs(np.sum(x * np.roll(y, -1, 1) - np.roll(x, -1, 1) * y, axis=1))


@pytest.mark.parametrize("orient", ["fluent", "random"])
def test_oracle_cell_nodes_quad_order(orient):
    """The reader's quad order (MshBlock.cpp:357-366) makes n0-n1 and n2-n3
    parallel: 0 1 2 3 is a bow tie, 0 1 3 2 the cyclic quad."""
    from mstcfd import meshgen as mg
    from oracle import pyoracle as po
    m = mg.reorient(mg.sod_strip(10, 2, ends=mg.OUTLET), orient, seed=1)
    om = po.mesh_from_arrays(m["node_xy"], m["face_nodes"], m["face_cells"], m["zones"],
                             m["n_cells"])
    ptr, ids = po.cell_nodes(om)
    assert np.all(np.diff(ptr) == 4)
    xy = om.node_xy[ids.reshape(-1, 4)]
    assert not np.any(np.isclose(_shoelace(xy), om.cell_vol))
    assert np.allclose(_shoelace(xy[:, [0, 1, 3, 2]]), om.cell_vol)


# ---------------------------------------------------------------------------
# GPU through the C ABI
# ---------------------------------------------------------------------------
def _solver(path, **kw):
    from mstcfd import Mesh, Solver
    mesh = Mesh.read_msh(path)
    return mesh, Solver(mesh, **kw)


@pytest.mark.gpu
@pytest.mark.parametrize("name", IO_CASES)
def test_gpu_plt_reference_mode_matches_golden(name, tmp_path):
    g = _golden()
    mesh, s = _solver(_msh(g, name, tmp_path), precision=0, reference_quirks=1)
    s.set_state(g[name + "_q"])
    out = os.path.join(str(tmp_path), "gpu.plt")
    s.write_plt(out, zone_t=7)
    assert open(out, "rb").read() == bytes(g[name + "_plt"])
    cell = os.path.join(str(tmp_path), "gpu.cell")
    s.write_cell_text(cell)
    assert open(cell, "rb").read() == bytes(g[name + "_cell"])
    s.read_cell_text(cell)
    assert np.array_equal(s.state(), g[name + "_readback"])


@pytest.mark.gpu
@pytest.mark.parametrize("quirks", [1, 0])
@pytest.mark.parametrize("prec", [0, 1, 2], ids=["exact", "fp64", "fp32"])
def test_gpu_node_values_match_oracle(quirks, prec):
    from mstcfd import Mesh, Solver
    from mstcfd import meshgen as mg
    from oracle import pyoracle as po
    m = mg.reorient(mg.tri_box(50, 30, 3.0, 2.0, jitter=0.25, seed=8), "random", seed=1)
    mesh = Mesh.from_arrays(m["node_xy"], m["face_nodes"], m["face_cells"], m["zones"],
                            m["n_cells"])
    om = po.mesh_from_arrays(m["node_xy"], m["face_nodes"], m["face_cells"], m["zones"],
                             m["n_cells"])
    s = Solver(mesh, precision=prec, reference_quirks=quirks)
    s.set_state(mg.random_state(mesh.n_cells, seed=5))
    q = s.state()  # the FP32 path holds the state as float pairs
    nq, nv = s.node_values()
    oq, ov = po.node_values(om, q, quirks=quirks, cv=715.8)
    assert np.array_equal(nq, oq)
    assert np.array_equal(nv, ov)


@pytest.mark.gpu
def test_gpu_plt_corrected_mode(tmp_path):
    from mstcfd import Mesh, Solver
    from mstcfd import meshgen as mg
    m = mg.tri_box(12, 7, 1.0, 0.6, jitter=0.2, seed=2)
    mesh = Mesh.from_arrays(m["node_xy"], m["face_nodes"], m["face_cells"], m["zones"],
                            m["n_cells"])
    s = Solver(mesh, reference_quirks=0)
    s.set_state(mg.random_state(mesh.n_cells, seed=1))
    out = os.path.join(str(tmp_path), "fixed.plt")
    s.write_plt(out, zone_t=4)
    lines = open(out).read().split("\n")
    assert lines[0] == 'TITLE = "Example: Variable and Connectivity List Sharing"'
    assert lines[2].endswith("ZONETYPE=FETRIANGLE")
    assert f"NODES={mesh.n_nodes}, ELEMENTS={mesh.n_cells}" in lines[2]
    conn = lines[3 + mesh.n_nodes:3 + mesh.n_nodes + mesh.n_cells]
    ids = np.array([[int(t) for t in ln.split()] for ln in conn])
    assert ids.shape == (mesh.n_cells, 3) and ids.min() == 1 and ids.max() == mesh.n_nodes
    vals = np.array([[float(t) for t in ln.split()] for ln in lines[3:3 + mesh.n_nodes]])
    nq, nv = s.node_values()
    assert np.allclose(vals[:, 2:], nv, rtol=0, atol=1e-15 * np.abs(nv).max())


@pytest.mark.gpu
def test_gpu_plt_corrected_mode_quads_cyclic(tmp_path):
    from mstcfd import Mesh, Solver
    from mstcfd import meshgen as mg
    m = mg.reorient(mg.sod_strip(20, 3, ends=mg.OUTLET), "random", seed=3)
    mesh = Mesh.from_arrays(m["node_xy"], m["face_nodes"], m["face_cells"], m["zones"],
                            m["n_cells"])
    s = Solver(mesh, reference_quirks=0)
    s.set_state(mg.random_state(mesh.n_cells, seed=1))
    out = os.path.join(str(tmp_path), "q.plt")
    s.write_plt(out)
    lines = open(out).read().split("\n")
    assert lines[2].endswith("ZONETYPE=FEQUADRILATERAL")
    nodes = np.array([[float(t) for t in ln.split()[:2]] for ln in lines[3:3 + mesh.n_nodes]])
    conn = lines[3 + mesh.n_nodes:3 + mesh.n_nodes + mesh.n_cells]
    ids = np.array([[int(t) for t in ln.split()] for ln in conn]) - 1
    vol = mesh.arrays()["cell_vol"]
    assert np.allclose(_shoelace(nodes[ids]), vol)


def _ckpt_case(prec):
    from mstcfd import Mesh, Solver
    from mstcfd import meshgen as mg
    m = mg.periodic_delaunay(40, 10.0, seed=6)
    mesh = Mesh.from_arrays(m["node_xy"], m["face_nodes"], m["face_cells"], m["zones"],
                            m["n_cells"], c1_shift=m["c1_shift"])
    arr = mesh.arrays()
    kw = dict(flux=0, order=2, limiter=2, reference_quirks=0, time_scheme=1, dt_mode=1,
              cfl=0.5, precision=prec)
    q0 = mg.isentropic_vortex(arr["cell_ctr"], length=10.0)
    return mesh, kw, q0, Solver


@pytest.mark.gpu
@pytest.mark.parametrize("prec", [0, 2], ids=["exact", "fp32"])
def test_gpu_checkpoint_restart_is_bitexact(prec, tmp_path):
    mesh, kw, q0, Solver = _ckpt_case(prec)
    a = Solver(mesh, **kw)
    a.set_state(q0)
    a.step(7)
    ck = os.path.join(str(tmp_path), "run.ckpt")
    a.checkpoint_save(ck)
    a.step(9)
    want, t_want = a.state(), a.time()
    b = Solver(mesh, **kw)
    b.checkpoint_load(ck)
    b.step(9)
    assert np.array_equal(b.state(), want)
    assert b.time() == t_want


@pytest.mark.gpu
def test_gpu_checkpoint_rejects_other_mesh_and_corruption(tmp_path):
    from mstcfd import Mesh, MstError, Solver
    from mstcfd import meshgen as mg
    mesh, kw, q0, _ = _ckpt_case(1)
    a = Solver(mesh, **kw)
    a.set_state(q0)
    ck = os.path.join(str(tmp_path), "a.ckpt")
    a.checkpoint_save(ck)
    # same cell count, other coordinates
    m2 = mg.periodic_delaunay(40, 10.0, seed=6)
    m2["node_xy"] = m2["node_xy"] * 1.0000001
    mesh2 = Mesh.from_arrays(m2["node_xy"], m2["face_nodes"], m2["face_cells"], m2["zones"],
                             m2["n_cells"], c1_shift=m2["c1_shift"])
    b = Solver(mesh2, **kw)
    with pytest.raises(MstError, match="another mesh"):
        b.checkpoint_load(ck)
    raw = bytearray(open(ck, "rb").read())
    raw[200] ^= 0x10
    bad = os.path.join(str(tmp_path), "bad.ckpt")
    open(bad, "wb").write(bytes(raw))
    with pytest.raises(MstError, match="checksum"):
        a.checkpoint_load(bad)
    open(bad, "wb").write(bytes(raw[:len(raw) // 2]))
    with pytest.raises(MstError):
        a.checkpoint_load(bad)
    with pytest.raises(MstError):
        a.read_cell_text(os.path.join(str(tmp_path), "missing.cellPUVT"))
