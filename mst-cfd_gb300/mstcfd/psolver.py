"""The reference's pressure-based SIMPLE solver on the GPU.

``PSolver`` mirrors the reference's PSolver (pSolver/PSolver.h:16-41) with
PSOLVER = SolverSIMPLE (pSolver/SolverSIMPLE.h:20-80), the solver the
reference's CONST.h selects with RHO_P 1: ``setDT``, ``solve`` (one time
step: SIMPLE_INTERVAL SIMPLE iterations), ``getNewValue`` /
``getOldValue`` / ``getOldNTimeValue`` and ``updateNewToOld``, on cell
states (p, u, v, T).  ``SimpleSolver.step(n)`` runs n time steps of the
reference's Time loop (time/Time.cpp:54-80) in one kernel launch.  Results
are bit-identical to the reference's SolverSIMPLE; there is no CPU path.
"""
import ctypes as C

import numpy as np

from . import capi


def default_params(**kw):
    p = capi.SimpleParams()
    capi.check(capi.load().mst_simple_default_params(C.byref(p)))
    for k, v in kw.items():
        if k == "inlet":
            for i in range(4):
                p.inlet[i] = float(v[i])
        else:
            setattr(p, k, v)
    return p


def q_to_puvt(q):
    """(p, u, v, T) of conserved states (Time::initialization)."""
    q = capi.f64(q).reshape(-1, 4)
    out = np.zeros_like(q)
    capi.check(capi.load().mst_q_to_puvt(len(q), capi.dptr(q), capi.dptr(out)))
    return out


def reference_initial(mesh, split_x=0.5):
    """The reference's initial field (time/Time.cpp:13-50): the uniform
    state of CONST.h in every cell, density x 0.125 and energy x 0.1 where
    the cell centre has x > split_x; every face starts from the uniform
    state.  Returns (cell PUVT, face PUVT)."""
    q0 = np.array([1.0, 0.0, 0.0, 1 * ((1 / 286.32) * 715.8 + 0.5 * (0 * 0 + 0 * 0))])
    ctr = mesh.arrays()["cell_ctr"]
    q = np.tile(q0, (mesh.n_cells, 1))
    right = ctr[:, 0] > split_x
    q[right, 0] *= 0.125
    q[right, 3] *= 0.1
    face = np.tile(q_to_puvt(q0[None])[0], (mesh.n_faces, 1))
    return q_to_puvt(q), face


class SimpleSolver:
    """SIMPLE time stepping of one mesh on the GPU."""

    def __init__(self, mesh, cell_puvt=None, face_puvt=None, **params):
        self.mesh = mesh
        self.params = default_params(**params)
        h = C.c_void_p()
        capi.check(capi.load().mst_simple_create(mesh._h, C.byref(self.params), C.byref(h)))
        self._h = h
        self.n_cells, self.n_faces = mesh.n_cells, mesh.n_faces
        if cell_puvt is None:
            cell_puvt, f0 = reference_initial(mesh)
            face_puvt = f0 if face_puvt is None else face_puvt
        self.set_state(cell_puvt, face_puvt)

    def set_state(self, cell_puvt, face_puvt=None):
        c = capi.f64(cell_puvt).reshape(self.n_cells, 4)
        f = None if face_puvt is None else capi.f64(face_puvt).reshape(self.n_faces, 4)
        capi.check(capi.load().mst_simple_set_state(
            self._h, capi.dptr(c), capi.dptr(f) if f is not None else None))

    def state(self):
        c = np.zeros((self.n_cells, 4))
        f = np.zeros((self.n_faces, 4))
        capi.check(capi.load().mst_simple_get_state(self._h, capi.dptr(c), capi.dptr(f)))
        return c, f

    def step(self, nsteps=1):
        """nsteps time steps; returns the Time loop's rows [nsteps][4]."""
        rows = np.zeros((max(int(nsteps), 1), 4))
        capi.check(capi.load().mst_simple_step(self._h, int(nsteps), capi.dptr(rows)))
        return rows[:nsteps]

    def rows(self):
        """SIMPLE iteration rows and Gauss-Seidel iteration counts of the
        last step() call."""
        i = self.info()
        n = max(i.last_steps, 1) * self.params.n_inner
        r = np.zeros((n, 4))
        g = np.zeros((n, 3), np.int32)
        capi.check(capi.load().mst_simple_rows(self._h, capi.dptr(r), capi.iptr(g)))
        k = i.last_steps
        return (r[:k * self.params.n_inner].reshape(k, -1, 4),
                g[:k * self.params.n_inner].reshape(k, -1, 3))

    def info(self):
        i = capi.SimpleInfo()
        capi.check(capi.load().mst_simple_get_info(self._h, C.byref(i)))
        return i

    def close(self):
        h = getattr(self, "_h", None)
        if h:
            capi.load().mst_simple_destroy(h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def step_batch(solvers, nsteps=1):
    """nsteps time steps of several SimpleSolvers in one launch (one
    thread-block cluster per case); returns their Time rows
    [n][nsteps][4]."""
    n = len(solvers)
    arr = (C.c_void_p * n)(*[s._h for s in solvers])
    rows = np.zeros((n, max(int(nsteps), 1), 4))
    capi.check(capi.load().mst_simple_step_batch(arr, n, int(nsteps), capi.dptr(rows)))
    return rows[:, :nsteps]


class PSolver:
    """The reference's PSolver call surface (pSolver/PSolver.h:16-41)."""

    def __init__(self, mesh, cell_puvt=None, face_puvt=None, **params):
        self._s = SimpleSolver(mesh, cell_puvt, face_puvt, **params)
        self._old_n = self._s.state()[0]

    def setDT(self, dt):
        cell, face = self._s.state()
        p = self._s.params
        self._s.close()
        self._s = SimpleSolver(self._s.mesh, cell, face, dt=float(dt), alpha_p=p.alpha_p,
                               n_inner=p.n_inner, wall_smooth=p.wall_smooth,
                               inlet=list(p.inlet), p_out=p.p_out, cluster=p.cluster)

    def solve(self):
        self._old_n = self._s.state()[0]
        self._s.step(1)

    def getNewValue(self):
        return self._s.state()[0]

    def getOldValue(self):
        return self._old_n

    def getOldNTimeValue(self):
        return self._old_n

    def updateNewToOld(self):
        """The step already leaves old = new (pSolver/PSolver.cpp:38-44)."""
