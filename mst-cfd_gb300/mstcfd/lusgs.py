"""The reference's sparse LU-SGS / Gauss-Seidel sweeps on the GPU.

``SparseSystem(block, dim, rows, cols, ops, vals)`` takes the matrix as the
ordered insertions the reference's SparseSolverNUM (setELE / addELE,
lusolver/SparseSolverNUM.cpp:115-140) or SparseSolver<Matrix4d, Vector4d>
(setD / setL / setU, lusolver/SparseSolver.cpp:35-48) would receive;
``solve(b, x0, method)`` runs solveILUSGS / solveGS / solveILU
level-scheduled on the GPU with results bit-identical to the reference's.
"""
import ctypes as C

import numpy as np

from . import capi


class SparseSystem:
    def __init__(self, block, dim, rows, cols, ops, vals):
        self.block, self.dim = int(block), int(dim)
        r = np.ascontiguousarray(rows, dtype=np.int32)
        c = np.ascontiguousarray(cols, dtype=np.int32)
        o = np.ascontiguousarray(ops if ops is not None else np.zeros(len(r)), dtype=np.int32)
        v = capi.f64(vals)
        h = C.c_void_p()
        capi.check(capi.load().mst_lu_create(self.block, self.dim, len(r), capi.iptr(r),
                                             capi.iptr(c), capi.iptr(o), capi.dptr(v),
                                             C.byref(h)))
        self._h = h

    def solve(self, b, x0, method=capi.LU_ILUSGS):
        b = capi.f64(b)
        x = capi.f64(x0).copy()
        it = C.c_int()
        capi.check(capi.load().mst_lu_solve(self._h, int(method), capi.dptr(b), capi.dptr(x),
                                            C.byref(it)))
        return x, it.value

    def levels(self):
        f, b = C.c_int(), C.c_int()
        capi.check(capi.load().mst_lu_levels(self._h, C.byref(f), C.byref(b)))
        return f.value, b.value

    def close(self):
        h = getattr(self, "_h", None)
        if h:
            capi.load().mst_lu_destroy(h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
