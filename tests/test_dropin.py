"""The C++ drop-in GpuRhoSolver (include/mstcfd_gpu_rhosolver.hpp).

* Against the reference's own headers (where they exist): the adapter
  compiles and links inside the reference build, in the time loop that
  Time::goNextTimeStep runs, with GpuRhoSolver in place of RhoSolver.
* On a GPU: the same time loop over stand-in classes with the reference's
  getters reproduces the reference's five-step states (golden) bit-for-bit.
"""
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT, golden_cases, golden_msh, load_golden

INC = os.path.join(ROOT, "include")
SHIM = os.path.join(ROOT, "oracle", "ref", "eigen_shim")
LIBDIR = os.path.join(ROOT, "mst-cfd_gb300", "lib")


def _lib():
    from mstcfd import capi
    capi.load()  # builds the library when missing
    return LIBDIR


@pytest.mark.ref
def test_dropin_builds_against_reference_headers(ref_available, tmp_path):
    from oracle import build
    src = os.path.join(build.REF_OUT, "ausm_o1", "src")
    objs = os.path.join(build.REF_OUT, "ausm_o1", "obj")
    ref_objs = [os.path.join(objs, f) for f in sorted(os.listdir(objs))
                if f.endswith(".o") and not f.startswith("harness")]
    exe = str(tmp_path / "dropin")
    cmd = ["g++", "-std=c++20", "-O2", "-fopenmp", "-ffp-contract=off", "-w",
           "-I", SHIM, "-I", src, "-I", INC,
           os.path.join(ROOT, "oracle", "ref", "harness_dropin.cpp")] + ref_objs + \
          ["-L", _lib(), "-lmstcfd", "-Wl,-rpath," + LIBDIR, "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    assert os.path.exists(exe)


@pytest.mark.gpu
@pytest.mark.parametrize("case", golden_cases(),
                         ids=[os.path.basename(c)[:-4] for c in golden_cases()])
def test_dropin_time_loop_matches_reference(case, tmp_path):
    from oracle import pyoracle as po
    g = load_golden(case)
    om = po.read_msh(golden_msh(g, tmp_path))
    exe = str(tmp_path / "standin")
    cmd = ["g++", "-std=c++20", "-O2", "-I", SHIM, "-I", INC,
           os.path.join(ROOT, "tests", "cpp", "dropin_standin.cpp"),
           "-L", _lib(), "-lmstcfd", "-Wl,-rpath," + LIBDIR, "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    nsteps = len(g["ausm_steps_log"])
    inp, out = str(tmp_path / "in.bin"), str(tmp_path / "out.bin")
    with open(inp, "wb") as f:
        np.array([om.n_nodes, om.n_cells, om.n_faces, len(om.zone), nsteps],
                 np.int32).tofile(f)
        om.node_xy.astype(np.float64).tofile(f)
        om.face_nodes.astype(np.int32).tofile(f)
        om.face_cells.astype(np.int32).tofile(f)
        om.zone.astype(np.int32).tofile(f)
        g["ausm_steps_q0"].astype(np.float64).tofile(f)
    r = subprocess.run([exe, inp, out], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    q = np.fromfile(out).reshape(-1, 4)
    assert np.array_equal(q, g["ausm_steps_q"], equal_nan=True)
