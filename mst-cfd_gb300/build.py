"""Builds the in-tree CUDA library ``mst-cfd_gb300/lib/libmstcfd.so``.

Translation units are compiled in parallel for sm_103a only:
  * csrc/mesh.cpp          host mesh front end (g++, -ffp-contract=off so the
                           geometry rounds like the reference on any host)
  * csrc/kernels_exact.cu  FP64 parity kernels, --fmad=false
  * csrc/kernels_fast.cu   FP64/FP32 production kernels (FMA allowed)
  * csrc/capi.cu           the C ABI of include/mstcfd.h
  * csrc/noalloc.cu        the allocation-free solve entry point
  * csrc/lusgs.cu          level-scheduled LU-SGS / GS sweeps, --fmad=false
  * csrc/simple.cu         the pressure-based SIMPLE solver, --fmad=false
  * csrc/io.cu             result writer (device node averaging) and
                           checkpoint files, --fmad=false
  * csrc/batch.cu          batched steady solves (LU-SGS orchestration,
                           CUDA graph, sweep autotuning)
  * csrc/mpnn.cu           the learned initial field (tcgen05 BF16 GEMMs)
  * csrc/mesh3d.cpp        3D solver geometry and device layout (g++,
                           -ffp-contract=off)
  * csrc/kernels3d_exact.cu / kernels3d_fast.cu   3D residual kernels
                           (FP64 parity without FMA; FP64 and FP32)
  * csrc/solver3d.cu       the 3D path's C ABI (mst_ctx3d_*)
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIBDIR = os.path.join(HERE, "lib")
LIB = os.path.join(LIBDIR, "libmstcfd.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc():
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _units():
    nv = _nvcc()
    common = ["-O3", "-std=c++17", "-lineinfo", "-I", INCLUDE,
              "-Xcompiler", "-fPIC,-ffp-contract=off"] + ARCH
    return [
        ("mesh.o", ["g++", "-O3", "-std=c++17", "-fPIC", "-ffp-contract=off",
                    "-Wall", "-c", os.path.join(CSRC, "mesh.cpp")]),
        ("kernels_exact.o", [nv] + common + ["--fmad=false", "-c",
                                             os.path.join(CSRC, "kernels_exact.cu")]),
        # single-precision division / square root to within 2 ulp and flush of
        # denormals on the production kernels (no effect on FP64 arithmetic)
        ("kernels_fast.o", [nv] + common + ["-prec-div=false", "-prec-sqrt=false",
                                            "-ftz=true", "-c",
                                            os.path.join(CSRC, "kernels_fast.cu")]),
        ("capi.o", [nv] + common + ["-c", os.path.join(CSRC, "capi.cu")]),
        ("noalloc.o", [nv] + common + ["-c", os.path.join(CSRC, "noalloc.cu")]),
        ("lusgs.o", [nv] + common + ["--fmad=false", "-c", os.path.join(CSRC, "lusgs.cu")]),
        ("simple.o", [nv] + common + ["--fmad=false", "-c", os.path.join(CSRC, "simple.cu")]),
        ("io.o", [nv] + common + ["--fmad=false", "-c", os.path.join(CSRC, "io.cu")]),
        ("batch.o", [nv] + common + ["-c", os.path.join(CSRC, "batch.cu")]),
        ("mpnn.o", [nv] + common + ["-c", os.path.join(CSRC, "mpnn.cu")]),
        ("mesh3d.o", ["g++", "-O3", "-std=c++17", "-fPIC", "-ffp-contract=off",
                      "-Wall", "-c", os.path.join(CSRC, "mesh3d.cpp")]),
        ("kernels3d_exact.o", [nv] + common + ["--fmad=false", "-c",
                                               os.path.join(CSRC, "kernels3d_exact.cu")]),
        ("kernels3d_fast.o", [nv] + common + ["-prec-div=false", "-prec-sqrt=false",
                                              "-ftz=true", "-c",
                                              os.path.join(CSRC, "kernels3d_fast.cu")]),
        ("solver3d.o", [nv] + common + ["-c", os.path.join(CSRC, "solver3d.cu")]),
    ]


def _deps():
    out = []
    for d in (CSRC, INCLUDE):
        for f in os.listdir(d):
            out.append(os.path.join(d, f))
    return out + [os.path.abspath(__file__)]


def build(force=False, verbose=False):
    """Compile (if stale) and return the path of libmstcfd.so."""
    if not force and os.path.exists(LIB):
        t = os.path.getmtime(LIB)
        if all(os.path.getmtime(p) <= t for p in _deps()):
            return LIB
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    units = _units()

    def run(u):
        name, cmd = u
        cmd = cmd + ["-o", os.path.join(OBJ, name)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        return name, r.returncode, r.stdout + r.stderr

    with ThreadPoolExecutor(max_workers=len(units)) as ex:
        results = list(ex.map(run, units))
    for name, rc, out in results:
        if verbose or rc:
            sys.stderr.write(f"--- {name} (rc={rc})\n{out}\n")
        if rc:
            raise RuntimeError(f"compiling {name} failed")
    tmp = LIB + ".tmp"
    link = [_nvcc(), "-shared"] + ARCH + ["-o", tmp] + \
        [os.path.join(OBJ, n) for n, _ in units]
    r = subprocess.run(link, capture_output=True, text=True)
    if r.returncode:
        raise RuntimeError("linking libmstcfd.so failed:\n" + r.stdout + r.stderr)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
