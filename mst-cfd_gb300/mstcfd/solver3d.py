"""The 3D residual path (mst_ctx3d_* of the C ABI): the 2D density path's
corrected mode carried to three dimensions -- Green-Gauss gradients,
split-axis Roe fluxes with limited MUSCL, the laminar viscous term, explicit
RK2 at a global CFL step -- on hand-written sm_103a kernels.  States are
[n_cells, 5] (rho, rho u, rho v, rho w, E) in file order."""
import ctypes as C

import numpy as np

from . import capi

PREC = {"exact": 0, "fp64": 1, "fp32": 2}


class Solver3D:
    def __init__(self, mesh, precision=2, order=2, limiter=3, viscous=0, mu=0.0, lambda_=None,
                 kappa=0.0, cv=1.0 / (1.4 * 0.4), inlet_q=None, cfl=0.5):
        p = capi.Params3D()
        capi.load().mst_params3d_default(C.byref(p))
        p.precision = PREC.get(precision, precision) if isinstance(precision, str) else precision
        p.order, p.limiter, p.viscous = int(order), int(limiter), int(viscous)
        p.mu = float(mu)
        p.lambda_ = float(-2.0 / 3.0 * mu if lambda_ is None else lambda_)
        p.kappa, p.cv, p.cfl = float(kappa), float(cv), float(cfl)
        if inlet_q is not None:
            for k in range(5):
                p.inlet_q[k] = float(inlet_q[k])
        h = C.c_void_p()
        capi.check(capi.load().mst_ctx3d_create(mesh._h, C.byref(p), C.byref(h)))
        self._h = h
        self.mesh = mesh
        i = capi.Ctx3DInfo()
        capi.check(capi.load().mst_ctx3d_info_get(self._h, C.byref(i)))
        self.info = {k: getattr(i, k) for k, _ in capi.Ctx3DInfo._fields_}
        self.n_cells = i.n_cells

    def set_state(self, q):
        q = np.ascontiguousarray(q, np.float64).reshape(self.n_cells, 5)
        capi.check(capi.load().mst_ctx3d_set_state(self._h, q.ctypes.data_as(capi._dp)))

    def state(self):
        q = np.zeros((self.n_cells, 5))
        capi.check(capi.load().mst_ctx3d_get_state(self._h, q.ctypes.data_as(capi._dp)))
        return q

    def residual(self):
        r = np.zeros((self.n_cells, 5))
        capi.check(capi.load().mst_ctx3d_residual(self._h, r.ctypes.data_as(capi._dp)))
        return r

    def gradient(self):
        g = np.zeros((self.n_cells, 3, 5))
        capi.check(capi.load().mst_ctx3d_gradient(self._h, g.ctypes.data_as(capi._dp)))
        return g

    def step(self, n=1, t_end=0.0):
        t = C.c_double()
        capi.check(capi.load().mst_ctx3d_step(self._h, int(n), float(t_end), C.byref(t)))
        return t.value

    def last_timing(self):
        ms, n = C.c_double(), C.c_int()
        capi.check(capi.load().mst_ctx3d_last_timing(self._h, C.byref(ms), C.byref(n)))
        return ms.value, n.value

    def kinetic_energy(self):
        ke, v = C.c_double(), C.c_double()
        capi.check(capi.load().mst_ctx3d_kinetic_energy(self._h, C.byref(ke), C.byref(v)))
        return ke.value, v.value

    def profile(self, on=True):
        capi.check(capi.load().mst_ctx3d_profile(self._h, 1 if on else 0))

    def profile_stats(self):
        L = capi.load()
        out = {}
        for i in range(L.mst_ctx3d_profile_count(self._h)):
            name = C.create_string_buffer(64)
            n, ms = C.c_int(), C.c_double()
            capi.check(L.mst_ctx3d_profile_get(self._h, i, name, 64, C.byref(n), C.byref(ms)))
            out[name.value.decode()] = (n.value, ms.value)
        return out

    def close(self):
        h = getattr(self, "_h", None)
        if h:
            capi.load().mst_ctx3d_destroy(h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
