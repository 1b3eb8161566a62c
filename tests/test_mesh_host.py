"""Product host mesh front end (C ABI, no GPU needed): reader and geometry
bit-exact against the reference (golden fixtures everywhere, the shipped
meshes where the reference exists), device renumbering invertible, and
malformed inputs rejected with status codes."""
import os

import numpy as np
import pytest

from conftest import golden_cases, golden_msh, load_golden, shipped_meshes

from mstcfd import Mesh, MstError, capi
from mstcfd import meshgen as mg

CASES = golden_cases()
IDS = [os.path.basename(c)[:-4] for c in CASES]
PAIRS = [("cell_vol", "cell_volume"), ("cell_ctr", "cell_center"),
         ("face_ctr", "face_center"), ("face_dir", "face_direct"),
         ("face_area", "face_area"), ("face_eta0", "face_eta0"),
         ("face_dac", "face_dac"), ("face_flag", "face_flag"),
         ("face_cells", "face_cells"), ("cell_ptr", "cell_ptr"),
         ("cell_faces", "cell_faces"), ("cell_nb", "cell_nbcells"),
         ("cell_dof", "cell_dof"), ("cell_eta0c", "cell_eta0c"),
         ("inner", "inner"), ("bond1", "bond1"), ("bond2", "bond2")]


def _eq(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return a.shape == b.shape and np.array_equal(a, b, equal_nan=a.dtype.kind == "f")


@pytest.mark.parametrize("case", CASES, ids=IDS)
def test_reader_matches_reference_golden(case, tmp_path):
    g = load_golden(case)
    a = Mesh.read_msh(golden_msh(g, tmp_path)).arrays()
    for mine, k in PAIRS:
        assert _eq(a[mine], g["geo_" + k]), mine


MESHES = shipped_meshes()


@pytest.mark.ref
@pytest.mark.parametrize("path", MESHES, ids=[os.path.basename(m) for m in MESHES])
def test_reader_matches_reference_shipped(ref_available, path):
    from oracle import refrun
    r = refrun.run(path, 0, 1)
    a = Mesh.read_msh(path).arrays()
    for mine, k in PAIRS:
        assert _eq(a[mine], getattr(r, k)), mine


@pytest.mark.parametrize("case", CASES, ids=IDS)
def test_from_arrays_matches_reader(case, tmp_path):
    from oracle import pyoracle as po
    g = load_golden(case)
    om = po.read_msh(golden_msh(g, tmp_path))
    a = Mesh.from_arrays(om.node_xy, om.face_nodes, om.face_cells, om.zone,
                         om.n_cells).arrays()
    for mine, k in PAIRS:
        assert _eq(a[mine], g["geo_" + k]), mine


def test_renumbering_is_a_permutation():
    m = mg.tri_box(40, 20, seed=9)
    a = Mesh.from_arrays(m["node_xy"], m["face_nodes"], m["face_cells"],
                         m["zones"], m["n_cells"]).arrays()
    for k, n in (("cell_perm", m["n_cells"]), ("face_perm", len(m["face_nodes"]))):
        p = a[k]
        assert np.array_equal(np.sort(p), np.arange(n)), k
        inv = np.empty_like(p)
        inv[p] = np.arange(n)
        assert np.array_equal(inv[p], np.arange(n))
    # the renumbering is not the identity on this mesh (Morton order)
    assert not np.array_equal(a["cell_perm"], np.arange(m["n_cells"]))


def test_crlf_and_lf_agree(tmp_path):
    m = mg.tri_box(12, 6, seed=2)
    p1, p2 = str(tmp_path / "a.msh"), str(tmp_path / "b.msh")
    mg.write_msh(p1, m, crlf=False)
    mg.write_msh(p2, m, crlf=True)
    a, b = Mesh.read_msh(p1).arrays(), Mesh.read_msh(p2).arrays()
    for k in a:
        assert _eq(a[k], b[k]), k


def test_periodic_mesh_closed():
    m = mg.periodic_delaunay(24, 10.0, seed=4)
    mesh = Mesh.from_arrays(m["node_xy"], m["face_nodes"], m["face_cells"],
                            m["zones"], m["n_cells"], c1_shift=m["c1_shift"])
    a = mesh.arrays()
    assert np.isclose(a["cell_vol"].sum(), 100.0, rtol=1e-12)
    # every cell is closed: the outward area vectors sum to zero
    s = np.add.reduceat(a["cell_dof"], a["cell_ptr"][:-1], axis=0)
    assert np.abs(s).max() < 1e-12
    assert np.all(a["face_dac"] == -1)  # generated "into c0"
    # centroids inside the fundamental domain
    assert a["cell_ctr"].min() >= -1e-9 and a["cell_ctr"].max() < 10.0 + 1e-9


BAD = {
    "truncated": lambda s: s[: len(s) // 2],
    # a face line whose cell id is past the cell count
    "bad_cell_id": lambda s: s.replace("\n1 ", "\nfffff ", 1).replace(
        s.split("(13 (3 1 ")[1].split("\n")[1], "1 2 fffff 1", 1),
    "no_faces": lambda s: "\n".join(l for l in s.split("\n") if not l.startswith("(13")),
    "blank_lines": lambda s: s.replace("\n", "\n\n", 40),
    "empty": lambda s: "",
}


@pytest.mark.parametrize("kind", sorted(BAD))
def test_malformed_msh_rejected(kind, tmp_path):
    m = mg.tri_box(6, 4, seed=1)
    p = str(tmp_path / "ok.msh")
    mg.write_msh(p, m)
    txt = BAD[kind](open(p).read())
    q = str(tmp_path / "bad.msh")
    open(q, "w").write(txt)
    with pytest.raises(MstError) as e:
        Mesh.read_msh(q)
    assert e.value.status in (capi.EMESH, capi.EINVAL)


def test_missing_file():
    with pytest.raises(MstError) as e:
        Mesh.read_msh("/nonexistent/mesh.msh")
    assert e.value.status == capi.EINVAL


def test_bad_arrays_rejected():
    m = mg.tri_box(6, 4, seed=1)
    z = m["zones"].copy()
    z[1, 1] += 1  # gap between zones
    with pytest.raises(MstError):
        Mesh.from_arrays(m["node_xy"], m["face_nodes"], m["face_cells"], z, m["n_cells"])
    fc = m["face_cells"].copy()
    fc[0, 0] = m["n_cells"] + 5
    with pytest.raises(MstError):
        Mesh.from_arrays(m["node_xy"], m["face_nodes"], fc, m["zones"], m["n_cells"])
