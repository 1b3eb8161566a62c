"""3D meshes (mst_mesh3d_* of the C ABI): the reader of MshBlock::readMsh
with DIM 3 and its reference geometry, or a mesh from arrays (generated,
optionally periodic); mstcfd.solver3d runs the 3D residual path on both."""
import ctypes as C
import os

import numpy as np

from . import capi


class Mesh3D:
    def __init__(self, path=None, _handle=None):
        h = _handle
        if h is None:
            h = C.c_void_p()
            capi.check(capi.load().mst_mesh3d_read_msh(os.fsencode(path), C.byref(h)))
        self._h = h
        i = capi.Mesh3DInfo()
        capi.check(capi.load().mst_mesh3d_get_info(self._h, C.byref(i)))
        self.info = {k: getattr(i, k) for k, _ in capi.Mesh3DInfo._fields_}
        self.n_cells, self.n_faces = i.n_cells, i.n_faces

    @classmethod
    def from_arrays(cls, node_xyz, faces, face_cells, zones, n_cells, c1_shift=None):
        """faces: [nF][3 or 4] array or a list of node lists (c0's frame for
        periodic faces); zones [nz][4] (id, first, last, type); c1_shift
        [nF][3] x(c0 frame) - x(c1 frame) or None."""
        if isinstance(faces, np.ndarray):
            ptr = np.arange(0, faces.size + 1, faces.shape[1], dtype=np.int32)
            fn = np.ascontiguousarray(faces.ravel(), np.int32)
        else:
            ptr = np.zeros(len(faces) + 1, np.int32)
            ptr[1:] = np.cumsum([len(f) for f in faces])
            fn = np.array([v for f in faces for v in f], np.int32)
        xyz = np.ascontiguousarray(node_xyz, np.float64)
        fc = np.ascontiguousarray(face_cells, np.int32)
        zn = np.ascontiguousarray(zones, np.int32).reshape(-1, 4)
        sh = None if c1_shift is None else np.ascontiguousarray(c1_shift, np.float64)
        h = C.c_void_p()
        capi.check(capi.load().mst_mesh3d_from_arrays(
            len(xyz), xyz.ctypes.data_as(capi._dp), int(n_cells), len(ptr) - 1,
            ptr.ctypes.data_as(capi._ip), fn.ctypes.data_as(capi._ip),
            fc.ctypes.data_as(capi._ip), len(zn), zn.ctypes.data_as(capi._ip),
            sh.ctypes.data_as(capi._dp) if sh is not None else None, C.byref(h)))
        return cls(_handle=h)

    @classmethod
    def from_dict(cls, m):
        """From a meshgen 3D mesh dict."""
        return cls.from_arrays(m["node_xyz"], m["faces"], m["face_cells"], m["zones"],
                               m["n_cells"], m.get("c1_shift"))

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
