"""Batched steady solves: many independent cases iterated together on one
GPU by matrix-free LU-SGS to a residual tolerance (mst_batch_* of the C
ABI).  Each case is a mesh with its own inflow state and transport
coefficients."""
import ctypes as C

import numpy as np

from . import capi

GAMMA = 1.4
PRANDTL = 0.72


def case_params(inlet_q, mu=0.0, lambda_=None, kappa=None, cv=1.0 / (GAMMA * (GAMMA - 1.0))):
    """Coefficients of one case; lambda = -2/3 mu and kappa = mu gamma cv /
    Pr by default (Stokes' hypothesis, Prandtl number 0.72)."""
    lam = -2.0 / 3.0 * mu if lambda_ is None else lambda_
    kap = mu * GAMMA * cv / PRANDTL if kappa is None else kappa
    return dict(inlet_q=np.asarray(inlet_q, float), mu=float(mu), lambda_=float(lam),
                kappa=float(kap), cv=float(cv))


def implicit_params(**kw):
    p = capi.ImplicitParams()
    capi.load().mst_implicit_params_default(C.byref(p))
    for k, v in kw.items():
        if not hasattr(p, k):
            raise KeyError(k)
        setattr(p, k, v)
    return p


class Batch:
    """cases: list of (Mesh, case_params dict); kw: mst_params fields of
    the residual (reference_quirks is forced to 0); implicit: dict of
    mst_implicit_params fields."""

    def __init__(self, cases, implicit=None, **kw):
        L = capi.load()
        self.meshes = [m for m, _ in cases]
        n = len(cases)
        arr = (C.c_void_p * n)(*[m._h for m in self.meshes])
        cps = (capi.CaseParams * n)()
        for i, (_, cp) in enumerate(cases):
            for k in range(4):
                cps[i].inlet_q[k] = float(cp["inlet_q"][k])
            cps[i].mu, cps[i].lambda_ = cp["mu"], cp["lambda_"]
            cps[i].kappa, cps[i].cv = cp["kappa"], cp["cv"]
        kw.setdefault("reference_quirks", 0)
        p = capi.params(**kw)
        ip = implicit_params(**(implicit or {}))
        h = C.c_void_p()
        capi.check(L.mst_batch_create(arr, cps, n, C.byref(p), C.byref(ip), C.byref(h)))
        self._h = h
        self.n_cases = n
        self.case_cells = np.cumsum([0] + [m.n_cells for m in self.meshes])

    def info(self):
        i = capi.BatchInfo()
        capi.check(capi.load().mst_batch_info(self._h, C.byref(i)))
        return {k: getattr(i, k) for k, _ in capi.BatchInfo._fields_}

    def colors(self):
        c = np.zeros(int(self.case_cells[-1]), np.int32)
        capi.check(capi.load().mst_batch_colors(self._h, c.ctypes.data_as(capi._ip)))
        return [c[a:b] for a, b in zip(self.case_cells[:-1], self.case_cells[1:])]

    def set_state(self, states):
        q = capi.f64(np.concatenate(states, 0), (int(self.case_cells[-1]), 4))
        capi.check(capi.load().mst_batch_set_state(self._h, capi.dptr(q)))

    def set_l2_ref(self, l2_ref):
        """Per-case reference L2 of the tolerance (after set_state); None
        clears it (the first iteration's L2 is the reference again)."""
        if l2_ref is None:
            capi.check(capi.load().mst_batch_set_l2_ref(self._h, None))
            return
        r = capi.f64(np.asarray(l2_ref, np.float64), (len(self.meshes),))
        capi.check(capi.load().mst_batch_set_l2_ref(self._h, capi.dptr(r)))

    def set_fallback(self, states):
        """Fallback state of every case (list of arrays, as set_state), or
        None: with stall_window set, a stalled case restarts from it."""
        if states is None:
            capi.check(capi.load().mst_batch_set_fallback(self._h, None))
            return
        q = capi.f64(np.concatenate(states, 0), (int(self.case_cells[-1]), 4))
        capi.check(capi.load().mst_batch_set_fallback(self._h, capi.dptr(q)))

    def restart(self, cases):
        """Restart the listed cases from their fallback states now."""
        ids = np.ascontiguousarray(cases, dtype=np.int32)
        capi.check(capi.load().mst_batch_restart(self._h, ids.ctypes.data_as(capi._ip), len(ids)))

    def state(self):
        q = np.zeros((int(self.case_cells[-1]), 4))
        capi.check(capi.load().mst_batch_get_state(self._h, capi.dptr(q)))
        return [q[a:b] for a, b in zip(self.case_cells[:-1], self.case_cells[1:])]

    def iterate(self, n):
        capi.check(capi.load().mst_batch_iterate(self._h, int(n)))

    def solve(self):
        r = capi.BatchResult()
        capi.check(capi.load().mst_batch_solve(self._h, C.byref(r)))
        return {k: getattr(r, k) for k, _ in capi.BatchResult._fields_}

    def case_status(self):
        n = self.n_cases
        it = np.zeros(n, np.int32)
        f, l = np.zeros(n), np.zeros(n)
        capi.check(capi.load().mst_batch_case_status(
            self._h, it.ctypes.data_as(capi._ip), capi.dptr(f), capi.dptr(l)))
        rs = np.zeros(n, np.int32)
        capi.check(capi.load().mst_batch_case_restarts(self._h, rs.ctypes.data_as(capi._ip)))
        return dict(conv_iter=it, first_l2=f, last_l2=l, restart_iter=rs)

    def close(self):
        h = getattr(self, "_h", None)
        if h:
            capi.load().mst_batch_destroy(h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def partition_cases(sizes, n_parts):
    """Greedy size balancing of independent cases over n_parts GPUs: cases
    in decreasing size, each to the currently lightest part (ties: the
    lowest part index).  Returns one sorted list of case indices per part.
    Cases never interact, so the parts need no exchange."""
    sizes = np.asarray(sizes, dtype=np.int64)
    load = np.zeros(int(n_parts), dtype=np.int64)
    parts = [[] for _ in range(int(n_parts))]
    for i in sorted(range(len(sizes)), key=lambda k: (-int(sizes[k]), k)):
        p = int(np.argmin(load))
        parts[p].append(i)
        load[p] += sizes[i]
    return [sorted(p) for p in parts]
