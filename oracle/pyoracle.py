"""ctypes wrapper of the C oracle ``mstoracle.c`` (test infrastructure only).

Arrays come back as numpy copies; the C mesh is freed when the Python object
is collected.  Layouts follow ``mstoracle.h``: states ``[n_cells, 4]``, face
flux matrices ``[n_faces, 2, 4]``, gradients ``[n_cells, 2, 4]``.
"""
import ctypes as C
import os

import numpy as np

from . import build as _build

AUSM, ROE = 0, 1

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_up = C.POINTER(C.c_uint8)


class _OMesh(C.Structure):
    _fields_ = [
        ("n_nodes", C.c_int), ("n_cells", C.c_int), ("n_faces", C.c_int),
        ("n_int_faces", C.c_int), ("n_zones", C.c_int),
        ("n_inner", C.c_int), ("n_bond1", C.c_int), ("n_bond2", C.c_int),
        ("zone", _ip), ("node_xy", _dp), ("face_nodes", _ip),
        ("face_cells", _ip), ("face_type", _ip), ("face_ctr", _dp),
        ("face_dir", _dp), ("face_area", _dp), ("face_eta0", _dp),
        ("face_dac", _ip), ("face_flag", _up), ("cell_ptr", _ip),
        ("cell_faces", _ip), ("cell_nb", _ip), ("cell_dof", _dp),
        ("cell_eta0c", _dp), ("cell_ctr", _dp), ("cell_vol", _dp),
        ("inner", _ip), ("bond1", _ip), ("bond2", _ip),
    ]


class _OParams(C.Structure):
    _fields_ = [("flux", C.c_int), ("order", C.c_int),
                ("inlet_q", C.c_double * 4)]


class _OParamsExt(C.Structure):
    _fields_ = [("flux", C.c_int), ("order", C.c_int), ("limiter", C.c_int),
                ("quirks", C.c_int), ("rk2", C.c_int), ("dt_mode", C.c_int),
                ("dt", C.c_double), ("cfl", C.c_double),
                ("inlet_q", C.c_double * 4), ("viscous", C.c_int), ("mu", C.c_double),
                ("lam", C.c_double), ("kappa", C.c_double), ("cv", C.c_double),
                ("phi", _dp), ("phi_mode", C.c_int), ("positivity", C.c_int)]


class _OLusgs(C.Structure):
    _fields_ = [("cfl0", C.c_double), ("cfl_max", C.c_double), ("omega", C.c_double),
                ("freeze_tol", C.c_double), ("tol", C.c_double), ("p_floor", C.c_double),
                ("refreeze_window", C.c_int)]


class _ONorms(C.Structure):
    _fields_ = [("linf", C.c_double * 4), ("l2", C.c_double * 4),
                ("mass", C.c_double), ("dt", C.c_double), ("time", C.c_double)]


_lib = None


class _OSimple(C.Structure):
    _fields_ = [("dt", C.c_double), ("alpha_p", C.c_double), ("n_inner", C.c_int),
                ("wall_smooth", C.c_int), ("inlet", C.c_double * 4),
                ("p_out", C.c_double)]


def lib():
    global _lib
    if _lib is None:
        path = _build.build_oracle()
        L = C.CDLL(path)
        L.om_mesh_read.argtypes = [C.c_char_p, C.POINTER(C.POINTER(_OMesh))]
        L.om_mesh_from_arrays.argtypes = [
            C.c_int, _dp, C.c_int, C.c_int, _ip, _ip, C.c_int, _ip,
            C.POINTER(C.POINTER(_OMesh))]
        L.om_mesh_free.argtypes = [C.POINTER(_OMesh)]
        L.om_default_params.argtypes = [C.POINTER(_OParams)]
        L.om_reference_inlet.argtypes = [_dp]
        for fn in ("om_ausm_flux", "om_roe_flux"):
            getattr(L, fn).argtypes = [_dp, _dp, C.c_int, _dp]
        L.om_gradient.argtypes = [C.POINTER(_OMesh), _dp, _dp, _dp]
        L.om_face_flux.argtypes = [C.POINTER(_OMesh), C.POINTER(_OParams),
                                   _dp, _dp, _dp]
        L.om_gather.argtypes = [C.POINTER(_OMesh), _dp, _dp]
        L.om_solve.argtypes = [C.POINTER(_OMesh), C.POINTER(_OParams), _dp,
                               C.c_double, _dp, _dp]
        L.om_linf_change.argtypes = [C.c_int, _dp, _dp, _dp]
        L.om_mesh_from_arrays_periodic.argtypes = [
            C.c_int, _dp, C.c_int, C.c_int, _ip, _ip, C.c_int, _ip, _dp,
            C.POINTER(C.POINTER(_OMesh))]
        L.om_default_params_ext.argtypes = [C.POINTER(_OParamsExt)]
        L.om_gradient_ext.argtypes = [C.POINTER(_OMesh), _dp, C.c_int, _dp]
        L.om_face_flux_ext.argtypes = [C.POINTER(_OMesh), C.POINTER(_OParamsExt),
                                       _dp, _dp, _dp]
        L.om_spectral_dt.argtypes = [C.POINTER(_OMesh), _dp, C.c_double, _dp]
        L.om_spectral_dt.restype = C.c_double
        L.om_step_ext.argtypes = [C.POINTER(_OMesh), C.POINTER(_OParamsExt), _dp,
                                  C.c_int, C.c_double, _dp, C.POINTER(_ONorms)]
        L.om_lu_scalar.argtypes = [C.c_int, C.c_int, C.c_int, _ip, _ip, _ip, _dp, _dp, _dp,
                                   _ip]
        L.om_lu_block.argtypes = [C.c_int, C.c_int, _ip, _ip, _dp, _dp, _dp]
        L.om_node_values.argtypes = [C.POINTER(_OMesh), _dp, C.c_int, C.c_double, _dp, _dp]
        L.om_cell_nodes.argtypes = [C.POINTER(_OMesh), _ip, _ip]
        L.om_write_plt.argtypes = [C.POINTER(_OMesh), _dp, C.c_double, C.c_int, C.c_char_p]
        L.om_write_cell_text.argtypes = [C.c_int, _dp, C.c_char_p]
        L.om_lusgs_iterate.argtypes = [C.POINTER(_OMesh), C.POINTER(_OParamsExt), _dp, _ip,
                                       C.POINTER(_OLusgs), C.c_int, _dp]
        L.om_greedy_colors.argtypes = [C.POINTER(_OMesh), _ip]
        L.om_simple_default_params.argtypes = [C.POINTER(_OSimple)]
        L.om_q_to_puvt.argtypes = [C.c_int, _dp, _dp]
        L.om_simple_step.argtypes = [C.POINTER(_OMesh), C.POINTER(_OSimple), _dp, _dp,
                                     C.c_int, _dp, _dp, _ip]
        _lib = L
    return _lib


def _d(a):
    return a.ctypes.data_as(_dp)


def _i(a):
    return a.ctypes.data_as(_ip)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


class Mesh:
    """Oracle mesh: the reference's MshBlock flattened to arrays."""

    def __init__(self, ptr):
        self._p = ptr
        m = ptr.contents
        self.n_nodes, self.n_cells = m.n_nodes, m.n_cells
        self.n_faces, self.n_int_faces = m.n_faces, m.n_int_faces
        nN, nC, nF, nZ = m.n_nodes, m.n_cells, m.n_faces, m.n_zones

        def arr(p, n, shape=None):
            a = np.ctypeslib.as_array(p, shape=(n,)).copy() if n else np.zeros(0)
            return a.reshape(shape) if shape else a

        self.zone = arr(m.zone, 4 * nZ, (nZ, 4))
        self.node_xy = arr(m.node_xy, 2 * nN, (nN, 2))
        self.face_nodes = arr(m.face_nodes, 2 * nF, (nF, 2))
        self.face_cells = arr(m.face_cells, 2 * nF, (nF, 2))
        self.face_type = arr(m.face_type, nF)
        self.face_ctr = arr(m.face_ctr, 2 * nF, (nF, 2))
        self.face_dir = arr(m.face_dir, 2 * nF, (nF, 2))
        self.face_area = arr(m.face_area, nF)
        self.face_eta0 = arr(m.face_eta0, nF)
        self.face_dac = arr(m.face_dac, nF)
        self.face_flag = arr(m.face_flag, 2 * nF, (nF, 2))
        self.cell_ptr = arr(m.cell_ptr, nC + 1)
        tot = int(self.cell_ptr[-1])
        self.cell_faces = arr(m.cell_faces, tot)
        self.cell_nb = arr(m.cell_nb, tot)
        self.cell_dof = arr(m.cell_dof, 2 * tot, (tot, 2))
        self.cell_eta0c = arr(m.cell_eta0c, tot)
        self.cell_ctr = arr(m.cell_ctr, 2 * nC, (nC, 2))
        self.cell_vol = arr(m.cell_vol, nC)
        self.inner = arr(m.inner, m.n_inner)
        self.bond1 = arr(m.bond1, m.n_bond1)
        self.bond2 = arr(m.bond2, m.n_bond2)

    def __del__(self):
        try:
            lib().om_mesh_free(self._p)
        except Exception:
            pass


def read_msh(path):
    p = C.POINTER(_OMesh)()
    rc = lib().om_mesh_read(os.fsencode(path), C.byref(p))
    if rc != 0:
        raise ValueError(f"oracle: cannot read mesh {path} (status {rc})")
    return Mesh(p)


def mesh_from_arrays(node_xy, face_nodes, face_cells, zones, n_cells,
                     c1_shift=None):
    node_xy = _f64(node_xy)
    fn = np.ascontiguousarray(face_nodes, dtype=np.int32)
    fc = np.ascontiguousarray(face_cells, dtype=np.int32)
    z = np.ascontiguousarray(zones, dtype=np.int32)
    sh = _f64(c1_shift) if c1_shift is not None else None
    p = C.POINTER(_OMesh)()
    rc = lib().om_mesh_from_arrays_periodic(
        len(node_xy), _d(node_xy), int(n_cells), len(fn), _i(fn), _i(fc),
        len(z), _i(z), _d(sh) if sh is not None else _dp(), C.byref(p))
    if rc != 0:
        raise ValueError(f"oracle: bad mesh arrays (status {rc})")
    return Mesh(p)


def params(flux=AUSM, order=1, inlet_q=None):
    p = _OParams()
    lib().om_default_params(C.byref(p))
    p.flux, p.order = flux, order
    if inlet_q is not None:
        for k in range(4):
            p.inlet_q[k] = float(inlet_q[k])
    return p


def reference_inlet():
    q = np.zeros(4)
    lib().om_reference_inlet(_d(q))
    return q


def riemann(flux, ql, qr, d):
    ql, qr = _f64(ql), _f64(qr)
    f = np.zeros(4)
    fn = lib().om_roe_flux if flux == ROE else lib().om_ausm_flux
    fn(_d(ql), _d(qr), int(d), _d(f))
    return f


def gradient(mesh, q):
    q = _f64(q)
    faceq = np.zeros((mesh.n_faces, 4))
    grad = np.zeros((mesh.n_cells, 2, 4))
    lib().om_gradient(mesh._p, _d(q), _d(faceq), _d(grad))
    return faceq, grad


def face_flux(mesh, prm, q, grad=None):
    q = _f64(q)
    F = np.zeros((mesh.n_faces, 2, 4))
    g = _d(_f64(grad)) if grad is not None else _dp()
    lib().om_face_flux(mesh._p, C.byref(prm), _d(q), g, _d(F))
    return F


def gather(mesh, F):
    F = _f64(F)
    R = np.zeros((mesh.n_cells, 4))
    lib().om_gather(mesh._p, _d(F), _d(R))
    return R


def solve(mesh, prm, q, dt):
    """One RhoSolver::solve(): returns (qnew, R)."""
    q = _f64(q)
    qn = np.zeros_like(q)
    R = np.zeros_like(q)
    lib().om_solve(mesh._p, C.byref(prm), _d(q), float(dt), _d(qn), _d(R))
    return qn, R


def linf_change(qold, qnew):
    qold, qnew = _f64(qold), _f64(qnew)
    r = np.zeros(4)
    lib().om_linf_change(len(qold), _d(qold), _d(qnew), _d(r))
    return r


# ---------------------------------------------------------------------------
# extensions (no reference counterpart): limiters, corrected boundaries,
# periodic images, CFL steps, two-stage Runge-Kutta
# ---------------------------------------------------------------------------
LIM_NONE, LIM_MINMOD, LIM_VANLEER, LIM_VANALBADA = range(4)
DT_FIXED, DT_CFL_GLOBAL, DT_CFL_LOCAL = range(3)


def params_ext(flux=AUSM, order=1, limiter=0, quirks=1, rk2=0, dt_mode=0,
               dt=1.0 / 4e3, cfl=0.5, inlet_q=None, viscous=0, mu=None, lam=None,
               kappa=None, cv=None):
    p = _OParamsExt()
    lib().om_default_params_ext(C.byref(p))
    p.flux, p.order, p.limiter, p.quirks, p.rk2 = flux, order, limiter, quirks, rk2
    p.dt_mode, p.dt, p.cfl = dt_mode, float(dt), float(cfl)
    p.viscous = int(viscous)
    for k, v in (("mu", mu), ("lam", lam), ("kappa", kappa), ("cv", cv)):
        if v is not None:
            setattr(p, k, float(v))
    if inlet_q is not None:
        for k in range(4):
            p.inlet_q[k] = float(inlet_q[k])
    return p


def gradient_ext(mesh, q, quirks):
    q = _f64(q)
    g = np.zeros((mesh.n_cells, 2, 4))
    lib().om_gradient_ext(mesh._p, _d(q), int(quirks), _d(g))
    return g


def face_flux_ext(mesh, prm, q, grad=None):
    q = _f64(q)
    F = np.zeros((mesh.n_faces, 2, 4))
    g = _d(_f64(grad)) if grad is not None else _dp()
    lib().om_face_flux_ext(mesh._p, C.byref(prm), _d(q), g, _d(F))
    return F


def spectral_dt(mesh, q, cfl):
    q = _f64(q)
    d = np.zeros(mesh.n_cells)
    m = lib().om_spectral_dt(mesh._p, _d(q), float(cfl), _d(d))
    return m, d


def step_ext(mesh, prm, q, nsteps, t_end=0.0, time=0.0):
    """nsteps steps; returns (q, norms dict of the last step)."""
    q = _f64(q).copy()
    t = C.c_double(time)
    n = _ONorms()
    rc = lib().om_step_ext(mesh._p, C.byref(prm), _d(q), int(nsteps), float(t_end),
                           C.byref(t), C.byref(n))
    if rc != 0:
        raise RuntimeError("om_step_ext failed")
    return q, dict(linf_change=np.array(n.linf[:]), l2_resid=np.array(n.l2[:]),
                   mass=n.mass, dt=n.dt, time=t.value)


# ---------------------------------------------------------------------------
# lusolver sweeps
# ---------------------------------------------------------------------------
def lu_scalar(gs, dim, rows, cols, ops, vals, b, x0):
    rows, cols, ops = (np.ascontiguousarray(a, dtype=np.int32) for a in (rows, cols, ops))
    vals, b = _f64(vals), _f64(b)
    x = _f64(x0).copy()
    it = C.c_int()
    lib().om_lu_scalar(int(gs), int(dim), len(rows), _i(rows), _i(cols), _i(ops), _d(vals),
                       _d(b), _d(x), C.byref(it))
    return x, it.value


def lu_block(dim, rows, cols, vals, b, x0):
    rows, cols = (np.ascontiguousarray(a, dtype=np.int32) for a in (rows, cols))
    vals, b = _f64(vals), _f64(b)
    x = _f64(x0).copy()
    lib().om_lu_block(int(dim), len(rows), _i(rows), _i(cols), _d(vals), _d(b), _d(x))
    return x


# ---------------------------------------------------------------------------
# result writer and text checkpoint (Work.cpp:204-319, :483-514)
# ---------------------------------------------------------------------------
def node_values(mesh, q, quirks=1, cv=715.8):
    """Node-averaged (node_q [nN][4], node_vars [nN][6] = rho u v T p Ma)."""
    q = _f64(q)
    nq = np.zeros((mesh.n_nodes, 4))
    nv = np.zeros((mesh.n_nodes, 6))
    rc = lib().om_node_values(mesh._p, _d(q), int(quirks), float(cv), _d(nq), _d(nv))
    if rc != 0:
        raise ValueError(f"oracle: node averaging refused (status {rc})")
    return nq, nv


def cell_nodes(mesh):
    ptr = np.zeros(mesh.n_cells + 1, np.int32)
    ids = np.zeros(4 * mesh.n_cells + 16, np.int32)
    lib().om_cell_nodes(mesh._p, _i(ptr), _i(ids))
    return ptr, ids[:ptr[-1]]


def write_plt(mesh, q, path, zone_t=0, cv=715.8):
    q = _f64(q)
    rc = lib().om_write_plt(mesh._p, _d(q), float(cv), int(zone_t), os.fsencode(path))
    if rc != 0:
        raise ValueError(f"oracle: cannot write {path} (status {rc})")


def write_cell_text(q, path):
    q = _f64(q)
    rc = lib().om_write_cell_text(len(q), _d(q), os.fsencode(path))
    if rc != 0:
        raise ValueError(f"oracle: cannot write {path} (status {rc})")


# ---------------------------------------------------------------------------
# implicit steady iterations (mstoracle_implicit.c)
# ---------------------------------------------------------------------------
def greedy_colors(mesh):
    col = np.zeros(mesh.n_cells, np.int32)
    n = lib().om_greedy_colors(mesh._p, _i(col))
    return col, n


def lusgs_iterate(mesh, prm, q, color, niter, cfl0=5.0, cfl_max=200.0, omega=1.5,
                  freeze_tol=0.0, tol=0.0, p_floor=0.0, refreeze_window=500):
    """niter LU-SGS iterations from q; returns (q, L2 history)."""
    q = _f64(q).copy()
    col = np.ascontiguousarray(color, dtype=np.int32)
    ip = _OLusgs(float(cfl0), float(cfl_max), float(omega), float(freeze_tol), float(tol),
                 float(p_floor), int(refreeze_window))
    hist = np.zeros(max(int(niter), 1))
    rc = lib().om_lusgs_iterate(mesh._p, C.byref(prm), _d(q), _i(col), C.byref(ip),
                                int(niter), _d(hist))
    if rc != 0:
        raise ValueError(f"oracle: lusgs failed (status {rc})")
    return q, hist[:int(niter)]


# ---------------------------------------------------------------------------
# 3D path (mstoracle3d.c): states [n_cells, 5], gradients [n_cells, 3, 5],
# face fluxes [n_faces, 3, 5]
# ---------------------------------------------------------------------------
class _O3Input(C.Structure):
    _fields_ = [("n_nodes", C.c_int), ("n_cells", C.c_int), ("n_faces", C.c_int),
                ("node_xyz", _dp), ("face_ptr", _ip), ("face_nodes", _ip),
                ("face_cells", _ip), ("face_type", _ip), ("c1_shift", _dp)]


class _O3Mesh(C.Structure):
    _fields_ = [("n_cells", C.c_int), ("n_faces", C.c_int), ("face_cells", _ip),
                ("face_kind", _ip), ("face_ctr", _dp), ("face_dir", _dp), ("r0", _dp),
                ("r1", _dp), ("eta", _dp), ("cell_ctr", _dp), ("cell_vol", _dp),
                ("cell_ptr", _ip), ("cell_faces", _ip), ("cell_nb", _ip), ("cell_dir", _dp),
                ("cell_w", _dp)]


class _O3Params(C.Structure):
    _fields_ = [("order", C.c_int), ("limiter", C.c_int), ("viscous", C.c_int),
                ("mu", C.c_double), ("lam", C.c_double), ("kappa", C.c_double),
                ("cv", C.c_double), ("inlet", C.c_double * 5)]


_lib3 = None


def lib3():
    global _lib3
    if _lib3 is None:
        L = lib()
        M = C.POINTER(_O3Mesh)
        L.om3_build.argtypes = [C.POINTER(_O3Input), M]
        L.om3_free.argtypes = [M]
        L.om3_gradient.argtypes = [M, _dp, _dp]
        L.om3_face_flux.argtypes = [M, C.POINTER(_O3Params), _dp, _dp, _dp]
        L.om3_gather.argtypes = [M, _dp, _dp]
        L.om3_residual.argtypes = [M, C.POINTER(_O3Params), _dp, _dp]
        L.om3_dt.argtypes = [M, _dp, C.c_double]
        L.om3_dt.restype = C.c_double
        L.om3_rk2.argtypes = [M, C.POINTER(_O3Params), _dp, C.c_int, C.c_double, C.c_double,
                              _dp]
        L.om3_kinetic_energy.argtypes = [M, _dp, _dp, _dp]
        _lib3 = L
    return _lib3


def _zone_types(zones, n_faces):
    t = np.zeros(n_faces, np.int32)
    for _, first, last, ty in np.asarray(zones).reshape(-1, 4).tolist():
        t[first - 1:last] = ty
    return t


class Mesh3:
    """Oracle 3D mesh: the solver geometry of mstoracle3d.c (file numbering)."""

    def __init__(self, node_xyz, faces, face_cells, zones, n_cells, c1_shift=None):
        faces = [list(f) for f in faces] if not isinstance(faces, np.ndarray) else faces
        if isinstance(faces, np.ndarray):
            ptr = np.arange(0, faces.size + 1, faces.shape[1], dtype=np.int32)
            fn = np.ascontiguousarray(faces.ravel(), np.int32)
        else:
            ptr = np.zeros(len(faces) + 1, np.int32)
            ptr[1:] = np.cumsum([len(f) for f in faces])
            fn = np.array([v for f in faces for v in f], np.int32)
        self._keep = [_f64(node_xyz), ptr, fn, np.ascontiguousarray(face_cells, np.int32),
                      _zone_types(zones, len(ptr) - 1)]
        shift = None if c1_shift is None else _f64(c1_shift)
        self._keep.append(shift)
        xyz, ptr, fn, fc, ft = self._keep[:5]
        inp = _O3Input(len(xyz), int(n_cells), len(ptr) - 1, _d(xyz), _i(ptr), _i(fn), _i(fc),
                       _i(ft), _d(shift) if shift is not None else None)
        self._m = _O3Mesh()
        if lib3().om3_build(C.byref(inp), C.byref(self._m)) != 0:
            raise ValueError("oracle: bad 3D mesh")
        self.n_cells = int(n_cells)
        self.n_faces = len(ptr) - 1

    def _arr(self, name, n, dt=np.float64):
        p = getattr(self._m, name)
        return np.ctypeslib.as_array(p, shape=(n,)).astype(dt).copy()

    def arrays(self):
        nF, nC = self.n_faces, self.n_cells
        tot = int(self._arr("cell_ptr", nC + 1, np.int64)[-1])
        return {"face_ctr": self._arr("face_ctr", 3 * nF).reshape(nF, 3),
                "face_dir": self._arr("face_dir", 3 * nF).reshape(nF, 3),
                "r0": self._arr("r0", 3 * nF).reshape(nF, 3),
                "r1": self._arr("r1", 3 * nF).reshape(nF, 3),
                "eta": self._arr("eta", nF),
                "face_kind": self._arr("face_kind", nF, np.int32),
                "cell_ctr": self._arr("cell_ctr", 3 * nC).reshape(nC, 3),
                "cell_vol": self._arr("cell_vol", nC),
                "cell_ptr": self._arr("cell_ptr", nC + 1, np.int32),
                "cell_faces": self._arr("cell_faces", tot, np.int32),
                "cell_nb": self._arr("cell_nb", tot, np.int32),
                "cell_dir": self._arr("cell_dir", 3 * tot).reshape(tot, 3)}

    def __del__(self):
        try:
            if getattr(self, "_m", None) is not None and _lib3 is not None:
                _lib3.om3_free(C.byref(self._m))
                self._m = None
        except Exception:
            pass


def params3(order=2, limiter=3, viscous=0, mu=0.0, lam=0.0, kappa=0.0, cv=1.0, inlet=None):
    p = _O3Params(int(order), int(limiter), int(viscous), float(mu), float(lam), float(kappa),
                  float(cv))
    if inlet is not None:
        for k in range(5):
            p.inlet[k] = float(inlet[k])
    return p


def gradient3(mesh, q):
    q = _f64(q)
    g = np.zeros((mesh.n_cells, 3, 5))
    lib3().om3_gradient(C.byref(mesh._m), _d(q), _d(g))
    return g


def face_flux3(mesh, prm, q, grad=None):
    q = _f64(q)
    F = np.zeros((mesh.n_faces, 3, 5))
    g = None if grad is None else _f64(grad)
    lib3().om3_face_flux(C.byref(mesh._m), C.byref(prm), _d(q), _d(g) if g is not None else None,
                         _d(F))
    return F


def gather3(mesh, F):
    F = _f64(F)
    R = np.zeros((mesh.n_cells, 5))
    lib3().om3_gather(C.byref(mesh._m), _d(F), _d(R))
    return R


def residual3(mesh, prm, q):
    q = _f64(q)
    R = np.zeros((mesh.n_cells, 5))
    lib3().om3_residual(C.byref(mesh._m), C.byref(prm), _d(q), _d(R))
    return R


def dt3(mesh, q, cfl):
    return float(lib3().om3_dt(C.byref(mesh._m), _d(_f64(q)), float(cfl)))


def rk2_3(mesh, prm, q, nsteps, cfl, t_end=0.0, time=0.0):
    """nsteps RK2 steps; returns (q, time)."""
    q = _f64(q).copy()
    t = C.c_double(time)
    if lib3().om3_rk2(C.byref(mesh._m), C.byref(prm), _d(q), int(nsteps), float(cfl),
                      float(t_end), C.byref(t)) != 0:
        raise ValueError("oracle: rk2 failed")
    return q, t.value


def kinetic_energy3(mesh, q):
    ke, v = C.c_double(), C.c_double()
    lib3().om3_kinetic_energy(C.byref(mesh._m), _d(_f64(q)), C.byref(ke), C.byref(v))
    return ke.value, v.value


# ---- pressure-based SIMPLE (mstoracle_simple.c) ----
def simple_params(**kw):
    p = _OSimple()
    lib().om_simple_default_params(C.byref(p))
    for k, v in kw.items():
        if k == "inlet":
            for i in range(4):
                p.inlet[i] = v[i]
        else:
            setattr(p, k, v)
    return p


def q_to_puvt(q):
    q = _f64(q).reshape(-1, 4)
    out = np.zeros_like(q)
    lib().om_q_to_puvt(len(q), _d(q), _d(out))
    return out


def simple_step(mesh, puvt, face, nsteps=1, prm=None):
    """nsteps SIMPLE time steps; returns (puvt, face, time rows, SIMPLE
    iteration rows, Gauss-Seidel iteration counts)."""
    prm = prm or simple_params()
    pv = _f64(puvt).reshape(-1, 4).copy()
    fc = _f64(face).reshape(-1, 4).copy()
    rows = np.zeros((nsteps, 4))
    inner = np.zeros((nsteps, prm.n_inner, 4))
    its = np.zeros((nsteps, prm.n_inner, 3), np.int32)
    rc = lib().om_simple_step(mesh._p, C.byref(prm), _d(pv), _d(fc), int(nsteps),
                              _d(rows), _d(inner), _i(its))
    if rc != 0:
        raise RuntimeError(f"om_simple_step failed ({rc})")
    return pv, fc, rows, inner, its
