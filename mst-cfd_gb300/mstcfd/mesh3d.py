"""3D Fluent meshes (mst_mesh3d_* of the C ABI): the reader of
MshBlock::readMsh with DIM 3 and its geometry, host only."""
import ctypes as C
import os

import numpy as np

from . import capi


class Mesh3D:
    def __init__(self, path):
        h = C.c_void_p()
        capi.check(capi.load().mst_mesh3d_read_msh(os.fsencode(path), C.byref(h)))
        self._h = h
        i = capi.Mesh3DInfo()
        capi.check(capi.load().mst_mesh3d_get_info(self._h, C.byref(i)))
        self.info = {k: getattr(i, k) for k, _ in capi.Mesh3DInfo._fields_}
        self.n_cells, self.n_faces = i.n_cells, i.n_faces

    def arrays(self):
        i = self.info
        nN, nC, nF = i["n_nodes"], i["n_cells"], i["n_faces"]
        tot, fn, cn = i["n_cell_faces"], i["n_face_nodes"], i["n_cell_nodes"]
        spec = dict(node_xyz=((nN, 3), np.float64), face_ptr=((nF + 1,), np.int32),
                    face_nodes=((fn,), np.int32), face_cells=((nF, 2), np.int32),
                    face_type=((nF,), np.int32), face_ctr=((nF, 3), np.float64),
                    face_dir=((nF, 3), np.float64), face_area=((nF,), np.float64),
                    face_eta0=((nF,), np.float64), face_cmd=((nF, 3), np.float64),
                    face_dac=((nF,), np.int32), face_flag=((nF, 3), np.uint8),
                    face_flag_set=((nF,), np.uint8), cell_ptr=((nC + 1,), np.int32),
                    cell_faces=((tot,), np.int32), cell_nb=((tot,), np.int32),
                    cell_dof=((tot, 3), np.float64), cell_eta0c=((tot,), np.float64),
                    cell_ctr=((nC, 3), np.float64), cell_vol=((nC,), np.float64),
                    cell_vol_fixed=((nC,), np.float64), cell_node_ptr=((nC + 1,), np.int32),
                    cell_nodes=((cn,), np.int32), inner=((i["n_inner"],), np.int32),
                    bond1=((i["n_bond1"],), np.int32), bond2=((i["n_bond2"],), np.int32),
                    cell_n_lower=((nC,), np.int32))
        out = {k: np.zeros(shape, dt) for k, (shape, dt) in spec.items()}
        a = capi.Mesh3DArrays()
        for k, v in out.items():
            ct = {np.float64: C.c_double, np.int32: C.c_int, np.uint8: C.c_uint8}[v.dtype.type]
            setattr(a, k, v.ctypes.data_as(C.POINTER(ct)) if v.size else None)
        capi.check(capi.load().mst_mesh3d_get_arrays(self._h, C.byref(a)))
        return out

    def close(self):
        h = getattr(self, "_h", None)
        if h:
            capi.load().mst_mesh3d_destroy(h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
