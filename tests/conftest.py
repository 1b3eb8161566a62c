import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "mst-cfd_gb300")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(ROOT, "tests", "golden")

def _ref_msh_dir():
    from oracle import build
    return os.path.join(build.REF_SRC, "msh")


REF_MSH_DIR = _ref_msh_dir()


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")
    config.addinivalue_line("markers", "ref: needs the reference sources (oracle/_ref)")


def _has_gpu():
    # A GPU machine exposes /dev/nvidia<N>; on one, GPU tests run and fail
    # loudly if the CUDA library is missing (no silent skip).
    import glob
    return bool(glob.glob("/dev/nvidia[0-9]*"))


HAS_GPU = _has_gpu()


def pytest_collection_modifyitems(config, items):
    skip_gpu = pytest.mark.skip(reason="no CUDA device")
    for it in items:
        if "gpu" in it.keywords and not HAS_GPU:
            it.add_marker(skip_gpu)


@pytest.fixture(scope="session")
def ref_available():
    from oracle import build
    if not build.ref_available():
        pytest.skip("reference sources not present on this machine")
    build.build_ref()
    return True


def shipped_meshes():
    if not os.path.isdir(REF_MSH_DIR):
        return []
    return sorted(os.path.join(REF_MSH_DIR, f) for f in os.listdir(REF_MSH_DIR)
                  if f.endswith(".msh"))


def golden_cases():
    import numpy as np
    out = []
    if os.path.isdir(GOLDEN):
        for f in sorted(os.listdir(GOLDEN)):
            if f.endswith(".npz") and not f.startswith(("lusolver", "writer", "simple",
                                                           "shipped")):
                out.append(os.path.join(GOLDEN, f))
    return out


def load_golden(path):
    import numpy as np
    with np.load(path, allow_pickle=False) as z:
        return {k: z[k] for k in z.files}


def golden_msh(g, tmp_path):
    """Write the golden case's mesh text to a file and return its path."""
    p = os.path.join(str(tmp_path), str(g["name"]) + ".msh")
    with open(p, "wb") as f:
        f.write(bytes(g["msh"]))
    return p
