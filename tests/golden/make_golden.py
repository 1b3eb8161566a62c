"""Generates the committed golden fixtures tests/golden/*.npz.

Each fixture is one generated mesh (written by mstcfd.meshgen.write_msh and
stored in the fixture as text) run through the REFERENCE ITSELF, compiled
from its own sources into oracle/_ref (oracle/ref/build_ref.sh):
  * the reference reader's geometry and connectivity (MshBlock),
  * one RhoSolver::solve() for AUSM+ and Roe at 1st order on a random
    physical state (sub- and supersonic) and at 2nd order on a smooth state
    (outlets retyped to walls, as the reference's 2nd-order outlet writes
    through unallocated pointers), with dt = 1e-3: per-face flux matrices,
    per-cell residuals, updated states,
  * five steps of the reference's own time loop (Time::goNextTimeStep with
    its Sod initialisation and DT = 1/4000) and the L-infinity residual rows
    it logs.
writer.npz: generated meshes with a random state, the Tecplot file and the
text checkpoint the reference's own Work members write for them
(oracle/ref/harness_io.cpp), and lusolver.npz: sparse systems with a mesh's sparsity, inserted in a
shuffled order (setELE/addELE mixed, duplicates kept), solved by the
reference's SparseSolverNUM::solveILUSGS / solveGS and
SparseSolver<Matrix4d, Vector4d>::solveILU (oracle/ref/harness_lu.cpp),
and simple.npz: generated meshes with inlet, outlet, wall and symmetry
zones run through the reference's pressure-based SolverSIMPLE
(oracle/ref/harness_simple.cpp: Time::initialization, then per step a
SolverSIMPLE solve with DT = 1/4000), from its own initial field and from
a random (p, u, v, T) state: the initial and final cell and face values,
the Time loop's residual rows and the Gauss-Seidel iteration counts.
The GPU tests compare the CUDA path against these arrays bit-for-bit on
machines where the reference is absent.

shipped.npz: two of the reference's shipped Fluent meshes (2d-stair-un-5-tri,
triangles; 2d-stair-st-2, quadrilaterals with 20 degenerate NaN-volume cells)
through the reference's solve() and time loop, outputs stored as SHA-256
digests (make_shipped).

Run from the repository root:  python tests/golden/make_golden.py
(only the shipped-mesh fixture:  python tests/golden/make_golden.py shipped)
"""
import os
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "mst-cfd_gb300"))

from mstcfd import meshgen as mg  # noqa: E402
from oracle import refrun  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))
DT = 1e-3
GEOM = ["face_cells", "face_dac", "face_center", "face_direct", "face_area",
        "face_eta0", "face_flag", "cell_ptr", "cell_faces", "cell_nbcells",
        "cell_dof", "cell_eta0c", "cell_center", "cell_volume", "inner",
        "bond1", "bond2", "zones"]


def cases():
    yield "tribox_mixed", mg.reorient(
        mg.tri_box(30, 15, 4.0, 2.0, jitter=0.2, seed=3), "random", seed=5)
    yield "quadstrip_fluent", mg.reorient(mg.sod_strip(24, 3, ends=mg.OUTLET), "fluent")
    yield "tribox_fluent", mg.reorient(
        mg.tri_box(10, 6, 1.0, 0.6, jitter=0.25, seed=7, left=mg.WALL,
                   right=mg.OUTLET, bottom=mg.SYMMETRY, top=mg.INLET), "fluent")


def make(name, mesh):
    d = tempfile.mkdtemp(prefix="golden_")
    msh = os.path.join(d, name + ".msh")
    mg.write_msh(msh, mesh, crlf=True)
    nC = int(mesh["n_cells"])
    out = {"name": np.array(name), "msh": np.frombuffer(open(msh, "rb").read(), np.uint8),
           "dt": np.array(DT)}
    q1 = mg.random_state(nC, seed=11)
    base = refrun.run(msh, 0, 1, q0=q1, dt=DT)
    for k in GEOM:
        out["geo_" + k] = getattr(base, k)
    out["q0_o1"] = base.q0
    q2 = mg.smooth_state(base.cell_center)
    out["q0_o2"] = q2
    for flux, fname in ((0, "ausm"), (1, "roe")):
        for order, q0 in ((1, q1), (2, q2)):
            r = refrun.run(msh, flux, order, q0=q0, dt=DT, remap5=(order == 2))
            v = f"{fname}_o{order}"
            out[v + "_flux"] = r.flux
            out[v + "_resid"] = r.resid
            out[v + "_qnew"] = r.qnew
        r = refrun.run(msh, flux, 1, time_steps=5)
        out[fname + "_steps_q0"] = r.q0
        out[fname + "_steps_q"] = r.q_steps
        out[fname + "_steps_log"] = r.time_log()
    path = os.path.join(OUT, name + ".npz")
    np.savez_compressed(path, **out)
    return path


def lu_system(dim_mesh, block, diag_scale, seed):
    """A sparse system with the sparsity of a triangle mesh's cell adjacency,
    inserted in a shuffled order with setELE/addELE mixed and some
    duplicated entries (the reference keeps duplicates)."""
    rng = np.random.default_rng(seed)
    m = mg.tri_box(*dim_mesh, seed=seed)
    fc = m["face_cells"]
    fc = fc[fc[:, 1] >= 0]
    dim = int(m["n_cells"])
    ins = [(int(a), int(b)) for a, b in fc] + [(int(b), int(a)) for a, b in fc]
    ins += [(i, i) for i in range(dim)]
    ins += [(i, i) for i in rng.choice(dim, dim // 5, replace=False)]  # repeated diagonal
    ins += [ins[i] for i in rng.choice(len(fc), len(fc) // 10, replace=False)]  # duplicates
    order = rng.permutation(len(ins))
    rows = np.array([ins[i][0] for i in order], np.int32)
    cols = np.array([ins[i][1] for i in order], np.int32)
    ops = rng.integers(0, 2, len(rows)).astype(np.int32)
    B = 16 if block else 1
    vals = rng.uniform(-1, 1, (len(rows), B))
    diag = rows == cols
    if block:
        eye = np.eye(4).ravel()
        vals[diag] = diag_scale * eye * rng.uniform(1, 1.5, (diag.sum(), 1)) + 0.2 * vals[diag]
    else:
        vals[diag, 0] = diag_scale * rng.uniform(1, 1.5, diag.sum())
    nb = 4 if block else 1
    b = rng.uniform(1, 2, dim * nb)
    x0 = rng.uniform(0.5, 1.5, dim * nb)
    return dim, rows, cols, ops, vals.ravel(), b, x0


def make_lu():
    out = {}
    specs = [("ilusgs", 0, (16, 10), False, 7.0, 31), ("ilusgs_fast", 0, (12, 8), False, 60.0, 32),
             ("gs", 1, (16, 10), False, 9.0, 33), ("gs_fast", 1, (12, 8), False, 80.0, 34),
             ("block", 2, (10, 8), True, 8.0, 35)]
    for name, mode, dm, block, ds, seed in specs:
        dim, rows, cols, ops, vals, b, x0 = lu_system(dm, block, ds, seed)
        x = refrun.run_lu(mode, dim, rows, cols, ops, vals, b, x0)
        for k, v in dict(dim=np.array(dim), mode=np.array(mode), rows=rows, cols=cols,
                         ops=ops, vals=vals, b=b, x0=x0, x=x).items():
            out[f"{name}_{k}"] = v
    path = os.path.join(OUT, "lusolver.npz")
    np.savez_compressed(path, **out)
    return path


def io_cases():
    yield "tri_iow", mg.reorient(mg.tri_box(16, 9, 1.0, 0.6, jitter=0.2, seed=3, left=mg.INLET,
                                           right=mg.OUTLET, bottom=mg.WALL, top=mg.WALL),
                                "random", seed=4)
    yield "quad_strip", mg.reorient(mg.sod_strip(24, 3, ends=mg.OUTLET), "fluent")


def make_io():
    out = {}
    for name, mesh in io_cases():
        d = tempfile.mkdtemp(prefix="golden_io_")
        msh = os.path.join(d, name + ".msh")
        mg.write_msh(msh, mesh, crlf=True)
        q = mg.random_state(int(mesh["n_cells"]), seed=21)
        plt, cell, back = refrun.run_io(msh, q, zone_t=7, time_now=5)
        out[name + "_msh"] = np.frombuffer(open(msh, "rb").read(), np.uint8)
        out[name + "_q"] = q
        out[name + "_plt"] = np.frombuffer(plt, np.uint8)
        out[name + "_cell"] = np.frombuffer(cell, np.uint8)
        out[name + "_readback"] = back
    path = os.path.join(OUT, "writer.npz")
    np.savez_compressed(path, **out)
    return path


def simple_cases():
    yield "tri_iow", mg.reorient(mg.tri_box(16, 9, 1.0, 0.6, jitter=0.2, seed=3, left=mg.INLET,
                                           right=mg.OUTLET, bottom=mg.WALL, top=mg.WALL),
                                "random", seed=4), 3
    yield "tri_sym", mg.reorient(
        mg.tri_box(12, 8, 1.0, 0.6, jitter=0.25, seed=9, left=mg.WALL, right=mg.OUTLET,
                   bottom=mg.SYMMETRY, top=mg.INLET), "fluent"), 3


def random_puvt(n, seed):
    rng = np.random.default_rng(seed)
    return np.stack([rng.uniform(0.5, 1.5, n), rng.uniform(-0.3, 0.3, n),
                     rng.uniform(-0.3, 0.3, n), rng.uniform(0.8, 1.2, n) / 286.32], 1)


def make_simple():
    out = {}
    for name, mesh, steps in simple_cases():
        d = tempfile.mkdtemp(prefix="golden_simple_")
        msh = os.path.join(d, name + ".msh")
        mg.write_msh(msh, mesh, crlf=True)
        out[name + "_msh"] = np.frombuffer(open(msh, "rb").read(), np.uint8)
        out[name + "_steps"] = np.array(steps)
        init = refrun.run_simple(msh, steps=0)
        r = refrun.run_simple(msh, steps=steps)
        out[name + "_init_puvt"] = init["puvt"]
        out[name + "_init_face"] = init["face"]
        for k in ("puvt", "face", "time_rows", "gs_iters"):
            out[f"{name}_init_{k}_out"] = r[k]
        p0 = random_puvt(int(mesh["n_cells"]), seed=41)
        r = refrun.run_simple(msh, puvt0=p0, steps=2)
        out[name + "_rand_puvt"] = p0
        for k in ("puvt", "face", "time_rows", "gs_iters"):
            out[f"{name}_rand_{k}_out"] = r[k]
    path = os.path.join(OUT, "simple.npz")
    np.savez_compressed(path, **out)
    return path


SHIPPED = ("2d-stair-un-5-tri", "2d-stair-st-2")


def digest(a):
    """SHA-256 of an FP64 array's bytes with every NaN made the same quiet
    NaN (CPU and GPU produce different NaN payloads)."""
    import hashlib
    a = np.ascontiguousarray(a, dtype=np.float64)
    a = np.where(np.isnan(a), np.float64("nan"), a)
    return hashlib.sha256(a.tobytes()).hexdigest()


def gentle_state(n, seed):
    """A state close to rest with small random variations (its 2nd-order
    reconstruction stays physical); from integer-exact random draws and
    IEEE arithmetic only, so any machine regenerates it bit for bit."""
    rng = np.random.default_rng(seed)
    return mg.primitive_to_q(1.0 + 0.05 * rng.uniform(-1, 1, n), 0.1 * rng.uniform(-1, 1, n),
                             0.1 * rng.uniform(-1, 1, n), 1.0 + 0.05 * rng.uniform(-1, 1, n))


def make_shipped():
    """Two of the reference's own Fluent meshes (msh/), run through the
    reference: one solve() for AUSM+ and Roe at 1st order on a random state
    and at 2nd order on a gentle state (outlets retyped to walls), and five
    steps of its time loop.  The meshes are stored; the outputs as digests
    (shipped meshes give large arrays), the initial states as the seeds of
    generators every machine reproduces exactly."""
    from oracle import build
    out = {"meshes": np.array(list(SHIPPED)), "dt": np.array(DT)}
    for name in SHIPPED:
        src = os.path.join(build.REF_SRC, "msh", name + ".msh")
        raw = open(src, "rb").read()
        out[name + "_msh"] = np.frombuffer(raw, np.uint8)
        d = tempfile.mkdtemp(prefix="golden_shipped_")
        msh = os.path.join(d, name + ".msh")
        with open(msh, "wb") as f:
            f.write(raw)
        base = refrun.run(msh, 0, 1, q0=None, dt=DT)
        nC = len(base.cell_volume)
        q1 = mg.random_state(nC, seed=11)
        q2 = gentle_state(nC, seed=12)
        out[name + "_q0_o1_sha"] = np.array(digest(q1))
        out[name + "_q0_o2_sha"] = np.array(digest(q2))
        for flux, fname in ((0, "ausm"), (1, "roe")):
            for order, q0 in ((1, q1), (2, q2)):
                r = refrun.run(msh, flux, order, q0=q0, dt=DT, remap5=(order == 2))
                v = f"{name}_{fname}_o{order}"
                out[v + "_resid_sha"] = np.array(digest(r.resid))
                out[v + "_qnew_sha"] = np.array(digest(r.qnew))
                out[v + "_resid_nan"] = np.array(int(np.isnan(r.resid).any(1).sum()))
            r = refrun.run(msh, flux, 1, time_steps=5)
            out[f"{name}_{fname}_steps_q0"] = r.q0
            out[f"{name}_{fname}_steps_q_sha"] = np.array(digest(r.q_steps))
            out[f"{name}_{fname}_steps_log"] = r.time_log()
    path = os.path.join(OUT, "shipped.npz")
    np.savez_compressed(path, **out)
    return path


if __name__ == "__main__":
    if sys.argv[1:] == ["shipped"]:
        p = make_shipped()
        print(p, os.path.getsize(p))
        sys.exit(0)
    for name, mesh in cases():
        p = make(name, mesh)
        print(p, os.path.getsize(p))
    p = make_lu()
    print(p, os.path.getsize(p))
    p = make_io()
    print(p, os.path.getsize(p))
    p = make_simple()
    print(p, os.path.getsize(p))
