"""The C ABI library loads without a GPU and exports every function that
include/*.h declares; host-only entry points work without a device."""
import ctypes as C
import glob
import os
import re

from conftest import ROOT

from mstcfd import capi


def _declared():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        txt = open(h).read()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        for m in re.finditer(r"^\s*[A-Za-z_][\w \*]*?\b(mst_\w+)\s*\(", txt, re.M):
            names.add(m.group(1))
    return names


def test_every_declared_symbol_is_exported():
    lib = capi.load()
    names = _declared()
    assert len(names) > 20
    missing = [n for n in sorted(names) if not hasattr(lib, n)]
    assert not missing, missing


def test_abi_version_and_defaults():
    lib = capi.load()
    assert lib.mst_abi_version() == 1
    p = capi.params()
    assert p.flux == capi.FLUX_AUSM and p.order == 1
    assert p.precision == capi.PREC_FP64_EXACT and p.reference_quirks == 1
    assert p.dt == 1.0 / 4e3
    from mstcfd import meshgen
    assert list(p.inlet_q) == list(meshgen.reference_inlet())


def test_null_arguments_return_status():
    lib = capi.load()
    assert lib.mst_mesh_read_msh(None, None) == capi.EINVAL
    assert lib.mst_solve(None) == capi.EINVAL
    assert lib.mst_step(None, 1, 0.0, None) == capi.EINVAL
    assert b"NULL" in lib.mst_last_error()
