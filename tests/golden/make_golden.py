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
The GPU tests compare the CUDA path against these arrays bit-for-bit on
machines where the reference is absent.

Run from the repository root:  python tests/golden/make_golden.py
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


if __name__ == "__main__":
    for name, mesh in cases():
        p = make(name, mesh)
        print(p, os.path.getsize(p))
