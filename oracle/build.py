"""Build steps for the oracle (test infrastructure only).

``build_oracle()`` compiles the C restatement ``mstoracle.c`` into
``oracle/_build/libmstoracle.so`` with ``-ffp-contract=off`` so every
operation rounds like the reference and the parity kernels.
``build_ref()`` runs ``ref/build_ref.sh`` when the reference checkout is
present (it is absent on machines that only run the prebuilt product).
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libmstoracle.so")
REF_OUT = os.path.join(HERE, "_ref")
# The reference checkout this build recipe compiles from: MSTCFD_REF_SRC,
# else the build container's read-only copy (absent on GPU machines, where
# build_ref() is a no-op).  The only place a path of the reference is named.
REF_SRC = os.environ.get("MSTCFD_REF_SRC") or "/root/reference/MST-CFD"

_SOURCES = ["mstoracle.c", "mstoracle_ext.c", "mstoracle_lu.c", "mstoracle_io.c",
            "mstoracle_simple.c",
            "mstoracle_implicit.c", "mstoracle3d.c"]


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build_oracle(force=False):
    os.makedirs(BUILD, exist_ok=True)
    srcs = [os.path.join(HERE, s) for s in _SOURCES if os.path.exists(os.path.join(HERE, s))]
    deps = srcs + [os.path.join(HERE, h) for h in
                   ("mstoracle.h", "mstoracle_io.h", "mstoracle_implicit.h", "mstoracle3d.h")]
    if force or _stale(LIB, deps):
        cmd = ["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-fopenmp",
               "-ffp-contract=off", "-Wall", "-o", LIB] + srcs + ["-lm"]
        subprocess.check_call(cmd)
    return LIB


def ref_available():
    return os.path.isfile(os.path.join(REF_SRC, "rhoSolver", "RhoSolver.cpp"))


def build_ref(force=False):
    """Compile the reference oracle binaries; returns False if the reference
    sources are not present on this machine."""
    if not ref_available():
        return False
    marker = os.path.join(REF_OUT, "ref_simple_mt")
    deps = [os.path.join(HERE, "ref", f) for f in
            ("build_ref.sh", "harness_rho.cpp", "harness_lu.cpp", "harness_io.cpp",
             "harness_mesh3d.cpp", "harness_simple.cpp",
             os.path.join("eigen_shim", "Eigen", "shim_matrix.h"))]
    if force or _stale(marker, deps):
        env = dict(os.environ, MSTCFD_REF_SRC=REF_SRC, MSTCFD_REF_OUT=REF_OUT)
        subprocess.check_call(["bash", os.path.join(HERE, "ref", "build_ref.sh")],
                              env=env, stdout=subprocess.DEVNULL)
    return True
