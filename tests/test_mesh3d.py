"""The 3D Fluent reader (mst_mesh3d_*; MshBlock::readMsh with DIM 3,
mesh/MshBlock.cpp:436-789), host only.

* against the reference's own reader built with DIM 3
  (oracle/ref/harness_mesh3d.cpp): every geometric and connectivity array
  bit-identical on jittered tetrahedra and hexahedra (left/right flags where
  the reference sets them);
* mixed-element zones (beyond the reference) read the same mesh as fixed
  zones; the corrected volumes sum to the box volume; malformed files fail
  with MST_EMESH.
"""
import os

import numpy as np
import pytest

PAIRS = [("node_xyz", "node_xyz"), ("face_ctr", "face_ctr"), ("face_dir", "face_dir"),
         ("face_area", "face_area"), ("face_eta0", "face_eta0"), ("face_cmd", "face_cmd"),
         ("face_dac", "face_dac"), ("face_cells", "face_cells"), ("face_ptr", "face_ptr"),
         ("face_nodes", "face_nodes"), ("cell_ctr", "cell_ctr"), ("cell_vol", "cell_vol"),
         ("cell_ptr", "cell_ptr"), ("cell_faces", "cell_faces"), ("cell_nb", "cell_nb"),
         ("cell_dof", "cell_dof"), ("cell_eta0c", "cell_eta0c"),
         ("cell_node_ptr", "cell_node_ptr"), ("cell_nodes", "cell_nodes"),
         ("cell_n_lower", "cell_nlow"), ("inner", "inner"), ("bond1", "bond1"),
         ("bond2", "bond2")]


def _meshes():
    from mstcfd import meshgen as mg
    return [("tet", mg.tet_box(4, jitter=0.15, seed=2)),
            ("hex", mg.hex_box(3, jitter=0.1, seed=4))]


@pytest.mark.ref
@pytest.mark.parametrize("case", [0, 1], ids=["tets", "hexes"])
def test_reader3d_matches_reference(ref_available, case, tmp_path):
    from mstcfd import meshgen as mg
    from mstcfd.mesh3d import Mesh3D
    from oracle import refrun
    name, m = _meshes()[case]
    p = os.path.join(str(tmp_path), name + ".msh")
    mg.write_msh3d(p, m, crlf=True)
    a = Mesh3D(p).arrays()
    r = refrun.run_mesh3d(p)
    for k, rk in PAIRS:
        assert np.array_equal(a[k].ravel(), r[rk].ravel()), k
    fs = a["face_flag_set"].astype(bool)
    assert fs.all()  # generated faces point into c0: the reference sets every flag
    assert np.array_equal(a["face_flag"][fs].ravel(), r["face_flag"].reshape(-1, 3)[fs].ravel())


def test_mixed_zones_and_corrected_volume(tmp_path):
    from mstcfd import meshgen as mg
    from mstcfd.mesh3d import Mesh3D
    m = mg.tet_box(3, jitter=0.15, seed=7)
    p1 = os.path.join(str(tmp_path), "fixed.msh")
    p2 = os.path.join(str(tmp_path), "mixed.msh")
    mg.write_msh3d(p1, m)
    mg.write_msh3d(p2, m, mixed_zones=tuple(range(len(m["zones"]))))
    a, b = Mesh3D(p1).arrays(), Mesh3D(p2).arrays()
    for k in a:
        assert np.array_equal(a[k], b[k]), k
    # tetrahedra have planar faces: the divergence-theorem volumes tile the box
    assert abs(a["cell_vol_fixed"].sum() - 1.0) < 1e-12
    assert np.all(a["cell_vol_fixed"] > 0)
    # the reference's formula (no 1/3, unsigned normals) does not
    assert abs(a["cell_vol"].sum() - 1.0) > 0.1


def test_reader3d_rejects_malformed(tmp_path):
    from mstcfd import MstError
    from mstcfd import meshgen as mg
    from mstcfd.mesh3d import Mesh3D
    m = mg.tet_box(2, seed=1)
    p = os.path.join(str(tmp_path), "ok.msh")
    mg.write_msh3d(p, m)
    text = open(p).read().split("\n")
    bad = os.path.join(str(tmp_path), "bad.msh")
    # a face line that names a cell beyond the total
    i = next(j for j, ln in enumerate(text) if ln.startswith("(13 (") and
             not ln.startswith("(13 (0 "))
    toks = text[i + 1].split()
    toks[-2] = "fff"
    text[i + 1] = " ".join(toks)
    open(bad, "w").write("\n".join(text))
    with pytest.raises(MstError):
        Mesh3D(bad)
    with pytest.raises(MstError):
        Mesh3D(os.path.join(str(tmp_path), "missing.msh"))
