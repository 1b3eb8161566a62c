"""mst_step_host_jobs: host-held states stepped through the device with the
copies on their own streams, overlapped with the computation.  Every job's
result must be bit-identical to the plain sequence set_state -> step ->
get_state of the same state (the same kernels run on the same data; only
the copies move to other streams), for the FP64 and the FP32 float-pair
paths, with page-locked and with ordinary host buffers."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec", [1, 2], ids=["fp64", "fp32"])
@pytest.mark.parametrize("pinned", [True, False], ids=["pinned", "pageable"])
def test_host_jobs_match_sequential_steps(prec, pinned):
    from mstcfd import Mesh, PinnedArray, Solver
    from mstcfd import meshgen as mg
    m = mg.periodic_delaunay(40, 10.0, seed=5)
    mesh = Mesh.from_arrays(m["node_xy"], m["face_nodes"], m["face_cells"], m["zones"],
                            m["n_cells"], c1_shift=m["c1_shift"])
    nC = mesh.n_cells
    base = mg.isentropic_vortex(m["cell_centroid"])
    states = [base * (1.0 + 0.01 * j) for j in range(5)]
    kw = dict(flux=0, order=2, limiter=2, reference_quirks=0, time_scheme=1, dt_mode=1,
              cfl=0.5, precision=prec)
    s = Solver(mesh, **kw)
    want = []
    for q in states:
        s.set_state(q)
        s.step(3)
        want.append(s.state())
    if pinned:
        ins = [PinnedArray((nC, 4)) for _ in states]
        outs = [PinnedArray((nC, 4)) for _ in states]
        for a, q in zip(ins, states):
            a.array[:] = q
        in_ptrs = [a.ptr.value for a in ins]
        out_ptrs = [a.ptr.value for a in outs]
        got = lambda j: outs[j].array  # noqa: E731
    else:
        ins = [np.ascontiguousarray(q) for q in states]
        outs = [np.zeros((nC, 4)) for _ in states]
        in_ptrs = [a.ctypes.data for a in ins]
        out_ptrs = [a.ctypes.data for a in outs]
        got = lambda j: outs[j]  # noqa: E731
    for rep in range(2):  # the second call reuses the pipeline's streams and slots
        s.step_host_jobs(in_ptrs, out_ptrs, nsteps=3)
        for j in range(len(states)):
            assert np.array_equal(got(j), want[j]), (rep, j)
    # the context holds the last job's result
    assert np.array_equal(s.state(), want[-1])
    s.close()
    if pinned:
        for a in ins + outs:
            a.free()


def test_host_jobs_argument_checks():
    from mstcfd import Mesh, Solver, capi
    from mstcfd import meshgen as mg
    import ctypes as C
    m = mg.tri_box(10, 6, 4.0, 2.0, jitter=0.2, seed=1)
    mesh = Mesh.from_arrays(m["node_xy"], m["face_nodes"], m["face_cells"], m["zones"],
                            m["n_cells"])
    s = Solver(mesh, dt=1e-4)
    L = capi.load()
    assert L.mst_step_host_jobs(None, 1, None, None, 1) == capi.EINVAL
    nul = (C.c_void_p * 1)(None)
    assert L.mst_step_host_jobs(s._h, 1, nul, nul, 1) == capi.EINVAL
    assert L.mst_step_host_jobs(s._h, 0, None, None, 1) == capi.OK
    s.close()
