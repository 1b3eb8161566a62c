"""Meshes and solver contexts over the C ABI.

``RhoSolver`` mirrors the reference's density-based solver surface
(rhoSolver/RhoSolver.h:14-56: setDT, solve, getOldValue, getNewValue,
updateNewToOld), with the state in and out as ``[n_cells, 4]`` arrays of
(rho, rho*u, rho*v, E) in the mesh file's cell numbering.
"""
import ctypes as C
import os

import numpy as np

from . import capi


class Mesh:
    """A mesh resident on the host; contexts upload it to the GPU."""

    def __init__(self, handle):
        self._h = handle
        info = capi.MeshInfo()
        capi.check(capi.load().mst_mesh_get_info(self._h, C.byref(info)))
        self.info = info
        self.n_cells, self.n_faces = info.n_cells, info.n_faces
        self.n_int_faces = info.n_int_faces
        self.n_nodes = info.n_nodes

    @classmethod
    def read_msh(cls, path):
        """Fluent ASCII 2D mesh (MshBlock::readMsh, mesh/MshBlock.cpp:5-18)."""
        h = C.c_void_p()
        capi.check(capi.load().mst_mesh_read_msh(os.fsencode(path), C.byref(h)))
        return cls(h)

    @classmethod
    def from_arrays(cls, node_xy, face_nodes, face_cells, zones, n_cells,
                    c1_shift=None):
        node_xy = capi.f64(node_xy)
        fn = np.ascontiguousarray(face_nodes, dtype=np.int32)
        fc = np.ascontiguousarray(face_cells, dtype=np.int32)
        z = np.ascontiguousarray(zones, dtype=np.int32)
        d = capi.MeshDesc()
        d.n_nodes, d.node_xy = len(node_xy), capi.dptr(node_xy)
        d.n_cells, d.n_faces = int(n_cells), len(fn)
        d.face_nodes, d.face_cells = capi.iptr(fn), capi.iptr(fc)
        d.n_zones, d.zones = len(z), capi.iptr(z)
        keep = [node_xy, fn, fc, z]
        if c1_shift is not None:
            sh = capi.f64(c1_shift)
            keep.append(sh)
            d.c1_shift = capi.dptr(sh)
        h = C.c_void_p()
        capi.check(capi.load().mst_mesh_create(C.byref(d), C.byref(h)))
        return cls(h)

    def arrays(self):
        """Host geometry in file numbering (for parity checks)."""
        i = self.info
        nF, nC, tot = i.n_faces, i.n_cells, i.n_cell_faces
        out = dict(
            face_ctr=np.zeros((nF, 2)), face_dir=np.zeros((nF, 2)),
            face_area=np.zeros(nF), face_eta0=np.zeros(nF),
            face_dac=np.zeros(nF, np.int32), face_flag=np.zeros((nF, 2), np.uint8),
            face_cells=np.zeros((nF, 2), np.int32),
            cell_ptr=np.zeros(nC + 1, np.int32), cell_faces=np.zeros(tot, np.int32),
            cell_nb=np.zeros(tot, np.int32), cell_dof=np.zeros((tot, 2)),
            cell_eta0c=np.zeros(tot), cell_ctr=np.zeros((nC, 2)),
            cell_vol=np.zeros(nC), inner=np.zeros(max(i.n_inner, 1), np.int32),
            bond1=np.zeros(max(i.n_bond1, 1), np.int32),
            bond2=np.zeros(max(i.n_bond2, 1), np.int32),
            cell_perm=np.zeros(nC, np.int32), face_perm=np.zeros(nF, np.int32))
        a = capi.MeshArrays()
        for name, arr in out.items():
            ptype = dict(capi.MeshArrays._fields_)[name]
            setattr(a, name, arr.ctypes.data_as(ptype))
        capi.check(capi.load().mst_mesh_get_arrays(self._h, C.byref(a)))
        out["inner"] = out["inner"][:i.n_inner]
        out["bond1"] = out["bond1"][:i.n_bond1]
        out["bond2"] = out["bond2"][:i.n_bond2]
        return out

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            try:
                capi.load().mst_mesh_destroy(h)
            except Exception:
                pass
            self._h = None


class Solver:
    """A device-resident solver context (one CUDA stream)."""

    def __init__(self, mesh, **kw):
        self.mesh = mesh
        self.p = capi.params(**kw)
        h = C.c_void_p()
        capi.check(capi.load().mst_ctx_create(mesh._h, C.byref(self.p), C.byref(h)))
        self._h = h
        self.n_cells = mesh.n_cells

    def set_params(self, **kw):
        for k, v in kw.items():
            if k == "inlet_q":
                for i in range(4):
                    self.p.inlet_q[i] = float(v[i])
            else:
                setattr(self.p, k, v)
        capi.check(capi.load().mst_ctx_set_params(self._h, C.byref(self.p)))

    def set_state(self, q):
        q = capi.f64(q, (self.n_cells, 4))
        capi.check(capi.load().mst_set_state(self._h, capi.dptr(q), 4))

    def state(self):
        q = np.zeros((self.n_cells, 4))
        capi.check(capi.load().mst_get_state(self._h, capi.dptr(q), 4))
        return q

    def new_state(self):
        q = np.zeros((self.n_cells, 4))
        capi.check(capi.load().mst_get_new_state(self._h, capi.dptr(q), 4))
        return q

    def residual(self):
        r = np.zeros((self.n_cells, 4))
        capi.check(capi.load().mst_get_residual(self._h, capi.dptr(r), 4))
        return r

    def face_flux(self):
        f = np.zeros((self.mesh.n_faces, 2, 4))
        capi.check(capi.load().mst_get_face_flux(self._h, capi.dptr(f)))
        return f

    def gradient(self):
        g = np.zeros((self.n_cells, 2, 4))
        capi.check(capi.load().mst_get_gradient(self._h, capi.dptr(g)))
        return g

    def set_dt(self, dt):
        capi.check(capi.load().mst_set_dt(self._h, float(dt)))
        self.p.dt = float(dt)

    def solve(self):
        capi.check(capi.load().mst_solve(self._h))

    def update_new_to_old(self):
        capi.check(capi.load().mst_update_new_to_old(self._h))

    def step(self, nsteps=1, t_end=0.0):
        n = capi.Norms()
        capi.check(capi.load().mst_step(self._h, int(nsteps), float(t_end), C.byref(n)))
        return dict(linf_change=np.array(n.linf_change[:]),
                    l2_resid=np.array(n.l2_resid[:]), dt=n.dt, time=n.time,
                    mass=n.mass)

    def time(self):
        t = C.c_double()
        capi.check(capi.load().mst_get_time(self._h, C.byref(t)))
        return t.value

    def last_timing(self):
        ms, n = C.c_double(), C.c_int()
        capi.check(capi.load().mst_last_timing(self._h, C.byref(ms), C.byref(n)))
        return ms.value, n.value

    def profile(self, on=True):
        capi.check(capi.load().mst_profile_enable(self._h, int(on)))

    def profile_reset(self):
        capi.check(capi.load().mst_profile_reset(self._h))

    def profile_stats(self):
        """{kernel name: (launches, total ms)} of the profiled launches."""
        L = capi.load()
        out = {}
        buf = C.create_string_buffer(128)
        for i in range(L.mst_profile_count(self._h)):
            n, ms = C.c_int(), C.c_double()
            capi.check(L.mst_profile_get(self._h, i, buf, 128, C.byref(n), C.byref(ms)))
            out[buf.value.decode()] = (n.value, ms.value)
        return out

    # -- result writer and checkpoints (work/Work.cpp:204-319, :432-514) --
    def node_values(self):
        """Node averages of the current state: (node_q [nN][4], node_vars
        [nN][6] = rho u v T p Ma), computed on the device."""
        n = self.mesh.n_nodes
        nq, nv = np.empty((n, 4)), np.empty((n, 6))
        capi.check(capi.load().mst_node_values(self._h, capi.dptr(nq), capi.dptr(nv)))
        return nq, nv

    def write_plt(self, path, zone_t=0):
        """Tecplot ASCII file of the current state (writedataRhoBasedMshNodePlt)."""
        capi.check(capi.load().mst_write_plt(self._h, os.fsencode(path), int(zone_t)))

    def write_cell_text(self, path):
        """Text checkpoint, 4 numbers per cell (writedataCellContinue)."""
        capi.check(capi.load().mst_write_cell_text(self._h, os.fsencode(path)))

    def read_cell_text(self, path):
        """State from a text checkpoint (readPbasedCellPlt)."""
        capi.check(capi.load().mst_read_cell_text(self._h, os.fsencode(path)))

    def checkpoint_save(self, path):
        """Exact binary checkpoint of state and time."""
        capi.check(capi.load().mst_checkpoint_save(self._h, os.fsencode(path)))

    def checkpoint_load(self, path):
        capi.check(capi.load().mst_checkpoint_load(self._h, os.fsencode(path)))

    def set_state_ptr(self, ptr, stride=4):
        """State in from a raw host pointer (e.g. a pinned buffer)."""
        capi.check(capi.load().mst_set_state(self._h, C.cast(ptr, capi._dp), stride))

    def get_state_ptr(self, ptr, stride=4):
        capi.check(capi.load().mst_get_state(self._h, C.cast(ptr, capi._dp), stride))

    def step_host_jobs(self, q_in_ptrs, q_out_ptrs, nsteps=1):
        """Independent host-held states (raw host pointers, [n_cells][4]
        doubles each; page-locked for full-speed copies) stepped nsteps
        each, copies overlapped with the computation."""
        n = len(q_in_ptrs)
        if len(q_out_ptrs) != n:
            raise ValueError("one output buffer per input")
        ins = (C.c_void_p * max(n, 1))(*[int(p) for p in q_in_ptrs])
        outs = (C.c_void_p * max(n, 1))(*[int(p) for p in q_out_ptrs])
        capi.check(capi.load().mst_step_host_jobs(self._h, n, ins, outs, int(nsteps)))

    def close(self):
        h = getattr(self, "_h", None)
        if h:
            capi.load().mst_ctx_destroy(h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class RhoSolver:
    """The reference's RhoSolver call surface on the GPU path.

    ``RhoSolver(mesh, state)`` plays ``RhoSolver(MshBlock*, fstream*,
    AllData*)``: ``state`` is a ``[n_cells, 4]`` array standing in for
    AllData's p1OldCellQs / p1NewCellQs.  As in the reference the solver
    reads the old state and writes the new state; ``updateNewToOld`` copies
    new into old.  Parameters default to the reference's (AUSM+, 1st order,
    DT = 1/4000) in the bit-exact FP64 arithmetic.
    """

    def __init__(self, mesh, state, **kw):
        self._s = Solver(mesh, **kw)
        self._state = state
        self._new = np.array(state, dtype=np.float64, copy=True)
        self._s.set_state(state)

    def setDT(self, dt):
        self._s.set_dt(dt)

    def solve(self):
        self._s.set_state(self._state)
        self._s.solve()
        self._new[:] = self._s.new_state()

    def getOldValue(self):
        return self._state

    def getNewValue(self):
        return self._new

    def updateNewToOld(self):
        self._state[:] = self._new

    def residual(self):
        return self._s.residual()


class PinnedArray:
    """A page-locked host array (mst_host_alloc) viewed through numpy."""

    def __init__(self, shape, dtype=np.float64):
        self.nbytes = int(np.prod(shape)) * np.dtype(dtype).itemsize
        self.ptr = C.c_void_p()
        capi.check(capi.load().mst_host_alloc(self.nbytes, C.byref(self.ptr)))
        buf = (C.c_char * self.nbytes).from_address(self.ptr.value)
        self.array = np.frombuffer(buf, dtype=dtype).reshape(shape)

    def free(self):
        if self.ptr:
            self.array = None
            capi.load().mst_host_free(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass
