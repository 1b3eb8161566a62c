"""Runs the reference compiled into oracle/_ref (test infrastructure only).

Only usable where the reference checkout exists (``build.ref_available()``);
tests that need it skip elsewhere and rely on the committed golden fixtures.
"""
import os
import subprocess
import tempfile

import numpy as np

from . import build as _build

VARIANTS = ("ausm_o1", "ausm_o2", "roe_o1", "roe_o2")


def variant(flux, order):
    return f"{'roe' if flux == 1 else 'ausm'}_o{order}"


class RefRun:
    """Outputs of one reference harness run (see oracle/ref/harness_rho.cpp)."""

    def __init__(self, outdir):
        self.dir = outdir

    def _load(self, name, dtype, shape=None):
        a = np.fromfile(os.path.join(self.dir, name), dtype=dtype)
        return a.reshape(shape) if shape else a

    def __getattr__(self, key):
        spec = {
            "counts": ("counts.i32", np.int32, None),
            "zones": ("zones.i32", np.int32, (-1, 4)),
            "nodes": ("nodes.f64", np.float64, (-1, 2)),
            "face_nodes": ("face_nodes.i32", np.int32, (-1, 2)),
            "face_cells": ("face_cells.i32", np.int32, (-1, 2)),
            "face_dac": ("face_dac.i32", np.int32, None),
            "face_type": ("face_type.i32", np.int32, None),
            "face_center": ("face_center.f64", np.float64, (-1, 2)),
            "face_direct": ("face_direct.f64", np.float64, (-1, 2)),
            "face_area": ("face_area.f64", np.float64, None),
            "face_eta0": ("face_eta0.f64", np.float64, None),
            "face_flag": ("face_flag.u8", np.uint8, (-1, 2)),
            "cell_ptr": ("cell_ptr.i32", np.int32, None),
            "cell_faces": ("cell_faces.i32", np.int32, None),
            "cell_nbcells": ("cell_nbcells.i32", np.int32, None),
            "cell_dof": ("cell_dof.f64", np.float64, (-1, 2)),
            "cell_eta0c": ("cell_eta0c.f64", np.float64, None),
            "cell_center": ("cell_center.f64", np.float64, (-1, 2)),
            "cell_volume": ("cell_volume.f64", np.float64, None),
            "bond_counts": ("bond_counts.i32", np.int32, None),
            "inner": ("inner.i32", np.int32, None),
            "bond1": ("bond1.i32", np.int32, None),
            "bond2": ("bond2.i32", np.int32, None),
            "q0": ("q0.f64", np.float64, (-1, 4)),
            "flux": ("flux.f64", np.float64, (-1, 2, 4)),
            "resid": ("resid.f64", np.float64, (-1, 4)),
            "qnew": ("qnew.f64", np.float64, (-1, 4)),
            "faceq": ("faceq.f64", np.float64, (-1, 4)),
            "q_steps": ("q_steps.f64", np.float64, (-1, 4)),
        }
        if key not in spec:
            raise AttributeError(key)
        return self._load(*spec[key])

    def time_log(self):
        """L-infinity residual rows the reference's Time loop logged."""
        rows = []
        with open(os.path.join(self.dir, "time.log")) as f:
            for line in f:
                if line.strip():
                    rows.append([float(x) for x in line.split()])
        return np.array(rows)


def run(mesh_path, flux=0, order=1, q0=None, dt=None, remap5=False,
        time_steps=0, outdir=None):
    """Run ref_rho_<variant> once; returns RefRun."""
    if not _build.build_ref():
        raise RuntimeError("reference sources not available")
    exe = os.path.join(_build.REF_OUT, "ref_rho_" + variant(flux, order))
    outdir = outdir or tempfile.mkdtemp(prefix="mstref_")
    args = [exe, os.path.abspath(mesh_path), outdir]
    if q0 is not None:
        qp = os.path.join(outdir, "q0_in.f64")
        np.ascontiguousarray(q0, dtype=np.float64).tofile(qp)
        args += ["--q0", qp]
    if dt is not None:
        args += ["--dt", repr(float(dt))]
    if remap5:
        args += ["--remap5to3"]
    if time_steps:
        args += ["--time-steps", str(int(time_steps))]
    subprocess.run(args, check=True, stdout=subprocess.DEVNULL,
                   stderr=subprocess.DEVNULL)
    return RefRun(outdir)


def run_lu(mode, dim, rows, cols, ops, vals, b, x0):
    """Run the reference lusolver harness (mode 0 ILU-SGS, 1 GS, 2 block)."""
    if not _build.build_ref():
        raise RuntimeError("reference sources not available")
    d = tempfile.mkdtemp(prefix="mstlu_")
    inp, out = os.path.join(d, "in.bin"), os.path.join(d, "out.bin")
    with open(inp, "wb") as f:
        np.array([mode, dim, len(rows)], np.int32).tofile(f)
        for a in (rows, cols, ops):
            np.ascontiguousarray(a, dtype=np.int32).tofile(f)
        for a in (vals, b, x0):
            np.ascontiguousarray(a, dtype=np.float64).tofile(f)
    subprocess.run([os.path.join(_build.REF_OUT, "ref_lu"), inp, out],
                   check=True, stdout=subprocess.DEVNULL)
    return np.fromfile(out, dtype=np.float64)


def run_io(mesh_path, q, zone_t=0, time_now=0):
    """Run the reference's writer members (oracle/ref/harness_io.cpp) on
    state q (file cell order).  Returns (plt bytes, cellPUVT bytes, the
    state readPbasedCellPlt reads back)."""
    if not _build.build_ref():
        raise RuntimeError("reference sources not available")
    d = tempfile.mkdtemp(prefix="mstio_")
    qp = os.path.join(d, "q_in.f64")
    np.ascontiguousarray(q, dtype=np.float64).tofile(qp)
    subprocess.run([os.path.join(_build.REF_OUT, "ref_io"), os.path.abspath(mesh_path), d, qp,
                    str(int(zone_t)), str(int(time_now))],
                   check=True, stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
    base = os.path.join(d, "result", f"mesh.msh_TIME4000_u0_t{int(time_now)}")
    with open(base + ".plt", "rb") as f:
        plt = f.read()
    with open(base + ".cellPUVT", "rb") as f:
        cell = f.read()
    back = np.fromfile(os.path.join(d, "readback.bin"), dtype=np.float64).reshape(-1, 4)
    return plt, cell, back


def run_simple(mesh_path, puvt0=None, steps=1, threads=1, bench=0):
    """The reference's SIMPLE solver (oracle/ref/harness_simple.cpp): dict
    with the cell and face (p, u, v, T) after ``steps`` time steps, the Time
    rows, the SIMPLE iteration rows and the Gauss-Seidel iteration counts
    (u, v, p' per SIMPLE iteration).  ``bench`` > 0: seconds per step."""
    if not _build.build_ref():
        raise RuntimeError("reference sources not available")
    exe = os.path.join(_build.REF_OUT, "ref_simple" if threads == 1 else "ref_simple_mt")
    d = tempfile.mkdtemp(prefix="mstsimple_")
    args = [exe, os.path.abspath(mesh_path), d]
    if puvt0 is not None:
        pp = os.path.join(d, "puvt0_in.f64")
        np.ascontiguousarray(puvt0, dtype=np.float64).tofile(pp)
        args += ["--puvt0", pp]
    if bench:
        r = subprocess.run(args + ["--bench", str(int(bench))], check=True,
                           capture_output=True, text=True)
        return float(r.stdout.strip().splitlines()[-1])
    subprocess.run(args + ["--steps", str(int(steps))], check=True,
                   stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
    out = dict(
        puvt=np.fromfile(os.path.join(d, "puvt.f64")).reshape(-1, 4),
        face=np.fromfile(os.path.join(d, "face_sc.f64")).reshape(-1, 4),
        time_rows=np.fromfile(os.path.join(d, "time_rows.f64")).reshape(-1, 4))
    with open(os.path.join(d, "time.log")) as f:
        out["inner_rows"] = np.array([[float(x) for x in ln.split()] for ln in f
                                      if ln.strip()])
    its, n = [], 0
    with open(os.path.join(d, "gs.log")) as f:
        for ln in f:
            if ln.startswith("LU-residual-GS"):
                k = int(ln.split()[1])
                if k == 0 and n:
                    its.append(n)
                n = k + 1
    if n:
        its.append(n)
    out["gs_iters"] = np.array(its, np.int32).reshape(-1, 3)
    return out


def run_mesh3d(mesh_path):
    """The reference's 3D reader (oracle/ref/harness_mesh3d.cpp): dict of
    its arrays."""
    if not _build.build_ref():
        raise RuntimeError("reference sources not available")
    d = tempfile.mkdtemp(prefix="mst3d_")
    subprocess.run([os.path.join(_build.REF_OUT, "ref_mesh3d"), os.path.abspath(mesh_path), d],
                   check=True, stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
    spec = {"counts": np.int32, "node_xyz": np.float64, "face_ctr": np.float64,
            "face_dir": np.float64, "face_area": np.float64, "face_eta0": np.float64,
            "face_cmd": np.float64, "face_dac": np.int32, "face_flag": np.uint8,
            "face_cells": np.int32, "face_ptr": np.int32, "face_nodes": np.int32,
            "cell_ctr": np.float64, "cell_vol": np.float64, "cell_ptr": np.int32,
            "cell_faces": np.int32, "cell_nb": np.int32, "cell_dof": np.float64,
            "cell_eta0c": np.float64, "cell_node_ptr": np.int32, "cell_nodes": np.int32,
            "cell_nlow": np.int32, "inner": np.int32, "bond1": np.int32, "bond2": np.int32}
    ext = {np.int32: "i32", np.float64: "f64", np.uint8: "u8"}
    return {k: np.fromfile(os.path.join(d, f"{k}.{ext[t]}"), dtype=t) for k, t in spec.items()}
