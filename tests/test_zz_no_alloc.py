"""mst_solve_device_noalloc: the allocation-free solve on caller-owned
device buffers, for programs that manage all device memory themselves and
cannot let the library call cudaMalloc/cudaFree while they run.

The test plays such a caller: it owns its device buffers (allocated here
through the CUDA runtime), calls the new entry point through the C ABI twice
in a row on the same buffers, and checks each call's new state, residual and
norms against the existing entry points (mst_solve / mst_step) on the same
input.  Tolerance: in FP64_EXACT the same kernels run in both, so states
and residuals must be identical (L2 norms to rtol 1e-12, mass to rtol 1e-13
as elsewhere in the GPU tests).  On the FP32 path mst_solve keeps the state
as float pairs while this entry point updates the caller's FP64 buffers, so
the two agree to FP32 rounding: the FP32 tolerances of the other tests
(residual within 2e-5 of its largest value per component, states within
1e-6 of theirs, norms to rtol 1e-5, and the mass to rtol 1e-9, since the
inlet and outlet fluxes that change it carry FP32 rounding).  Kept in its own file, collected
last, so a run that stops at the first failure has run every other test.
"""
import ctypes as C
import ctypes.util
import glob
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _cudart():
    cands = [ctypes.util.find_library("cudart")]
    cands += sorted(glob.glob("/usr/local/cuda/lib64/libcudart.so*"))
    cands += sorted(glob.glob("/usr/local/cuda/targets/*/lib/libcudart.so*"))
    for c in cands:
        if not c:
            continue
        try:
            rt = C.CDLL(c)
        except OSError:
            continue
        rt.cudaMalloc.argtypes = [C.POINTER(C.c_void_p), C.c_size_t]
        rt.cudaFree.argtypes = [C.c_void_p]
        rt.cudaMemcpy.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_int]
        rt.cudaMemGetInfo.argtypes = [C.POINTER(C.c_size_t), C.POINTER(C.c_size_t)]
        return rt
    pytest.fail("CUDA runtime library not found")


class _DevBuf:
    """A device buffer owned by the caller (cudaMalloc is 256-byte aligned)."""

    def __init__(self, rt, nbytes):
        self.rt, self.n = rt, nbytes
        self.p = C.c_void_p()
        assert rt.cudaMalloc(C.byref(self.p), nbytes) == 0

    def put(self, a):
        a = np.ascontiguousarray(a, dtype=np.float64)
        assert a.nbytes == self.n
        assert self.rt.cudaMemcpy(self.p, a.ctypes.data, self.n, 1) == 0

    def get(self, shape):
        out = np.empty(shape, dtype=np.float64)
        assert self.rt.cudaMemcpy(out.ctypes.data, self.p, self.n, 2) == 0
        return out

    def free(self):
        self.rt.cudaFree(self.p)


_VISC = dict(viscous=1, mu=0.02, lambda_=-2.0 / 3.0 * 0.02, kappa=0.03, cv=2.5)
_CASES = {
    "fp64_exact-o1": (0, 1, {}),
    "fp64_exact-o2": (0, 2, {}),
    "fp32-o1": (2, 1, {}),
    "fp32-o2": (2, 2, {}),
    "fp64-o2": (1, 2, {}),
    "fp64-minmod": (1, 2, dict(limiter=1, reference_quirks=0)),
    "fp64_exact-vanleer-viscous": (0, 2, dict(limiter=2, reference_quirks=0, **_VISC)),
    "fp32-vanleer-viscous": (2, 2, dict(limiter=2, reference_quirks=0, **_VISC)),
}


def _free_bytes(rt):
    free, total = C.c_size_t(), C.c_size_t()
    assert rt.cudaMemGetInfo(C.byref(free), C.byref(total)) == 0
    return free.value


@pytest.mark.parametrize("case", list(_CASES))
def test_noalloc_matches_existing_entry_points(case):
    from mstcfd import Mesh, Solver, capi
    from mstcfd import meshgen as mg
    prec, order, kw = _CASES[case]
    m = mg.reorient(mg.tri_box(60, 30, 4.0, 2.0, jitter=0.25, seed=44), "random", seed=2)
    if order == 2:
        m = mg.with_zone_types(m, mg.OUTLET, mg.WALL)
    mesh = Mesh.from_arrays(m["node_xy"], m["face_nodes"], m["face_cells"], m["zones"],
                            m["n_cells"])
    arrs = mesh.arrays()
    q0 = mg.smooth_state(arrs["cell_ctr"])
    s = Solver(mesh, order=order, precision=prec, dt=2e-4, **kw)
    # existing entry points
    s.set_state(q0)
    s.solve()
    want_qn, want_r = s.new_state(), s.residual()
    s.set_state(q0)
    want_norms = s.step(1)
    # the caller's own device buffers, rows in the context's device order
    nC = mesh.n_cells
    perm = arrs["cell_perm"]
    q_dev_order = np.empty_like(q0)
    q_dev_order[perm] = q0
    rt = _cudart()
    bq, bqn, br = (_DevBuf(rt, nC * 32) for _ in range(3))
    bn = _DevBuf(rt, 10 * 8)
    try:
        bq.put(q_dev_order)
        lib = capi.load()
        for call in range(2):
            free0 = _free_bytes(rt)
            st = lib.mst_solve_device_noalloc(s._h, bq.p, bqn.p, br.p, bn.p)
            assert st == capi.OK, lib.mst_last_error()
            if call == 1:
                # the point of the entry point: no device memory taken by the call
                assert _free_bytes(rt) == free0
            qn = bqn.get((nC, 4))[perm]
            r = br.get((nC, 4))[perm]
            nrm = bn.get(10)
            if prec in (0, 1):
                assert np.array_equal(qn, want_qn), call
                assert np.array_equal(r, want_r), call
                assert np.array_equal(nrm[:4], want_norms["linf_change"]), call
                assert np.allclose(nrm[4:8], want_norms["l2_resid"], rtol=1e-12, atol=0), call
                assert np.isclose(nrm[8], want_norms["mass"], rtol=1e-13, atol=0), call
            else:
                scale = np.abs(want_r).max(0)
                assert np.all(np.abs(r - want_r).max(0) <= 2e-5 * scale), call
                assert np.all(np.abs(qn - want_qn) <= 1e-6 * np.abs(want_qn).max(0)), call
                assert np.allclose(nrm[:8], np.concatenate([want_norms["linf_change"],
                                                             want_norms["l2_resid"]]),
                                   rtol=1e-5, atol=0), call
                assert np.isclose(nrm[8], want_norms["mass"], rtol=1e-9, atol=0), call
            assert nrm[9] == want_norms["dt"], call
    finally:
        for b in (bq, bqn, br, bn):
            b.free()
        s.close()


def test_noalloc_rejects_meshes_over_the_limit():
    from mstcfd import Mesh, Solver, capi
    from mstcfd import meshgen as mg
    m = mg.tri_box(300, 240, 4.0, 2.0, jitter=0.2, seed=5)
    assert m["n_cells"] > 131072
    mesh = Mesh.from_arrays(m["node_xy"], m["face_nodes"], m["face_cells"], m["zones"],
                            m["n_cells"])
    s = Solver(mesh, dt=1e-4)
    rt = _cudart()
    b = _DevBuf(rt, mesh.n_cells * 32)
    try:
        lib = capi.load()
        st = lib.mst_solve_device_noalloc(s._h, b.p, b.p, None, None)
        assert st == capi.EINVAL
        assert b"at most 131072" in lib.mst_last_error()
    finally:
        b.free()
        s.close()


def test_noalloc_rejects_overlap_and_multi_stage_contexts():
    from mstcfd import Mesh, Solver, capi
    from mstcfd import meshgen as mg
    m = mg.tri_box(20, 10, 4.0, 2.0, jitter=0.2, seed=6)
    mesh = Mesh.from_arrays(m["node_xy"], m["face_nodes"], m["face_cells"], m["zones"],
                            m["n_cells"])
    rt = _cudart()
    nb = mesh.n_cells * 32
    b = _DevBuf(rt, 3 * nb)
    lib = capi.load()
    try:
        s = Solver(mesh, dt=1e-4)
        q = b.p.value
        # the new state may not alias the input, nor the residual either one
        assert lib.mst_solve_device_noalloc(s._h, q, q, None, None) == capi.EINVAL
        assert b"must not overlap" in lib.mst_last_error()
        assert lib.mst_solve_device_noalloc(s._h, q, q + nb, q + 32, None) == capi.EINVAL
        assert lib.mst_solve_device_noalloc(s._h, q, q + nb, q + 2 * nb, None) == capi.OK
        s.close()
        # two RK stages or a CFL step are not what one call does: refused
        for kw in (dict(time_scheme=1), dict(dt_mode=1, cfl=0.5)):
            s = Solver(mesh, dt=1e-4, **kw)
            st = lib.mst_solve_device_noalloc(s._h, q, q + nb, None, None)
            assert st == capi.EUNSUPPORTED, kw
            s.close()
    finally:
        b.free()
