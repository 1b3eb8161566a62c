"""The reference's lusolver sweeps: oracle and GPU against the reference.

* oracle (C restatement) against the fixtures the reference's own
  SparseSolverNUM / SparseSolver produced (tests/golden/lusolver.npz), and
  against the reference binary on fresh random systems where it exists;
* GPU (level-scheduled, through the C ABI) against the same fixtures and
  against the oracle on larger mesh-sparsity systems: bit-for-bit, and the
  same number of outer iterations (the reference's early exit included).
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN

from oracle import pyoracle as po

NAMES = ["ilusgs", "ilusgs_fast", "gs", "gs_fast", "block"]


def _case(name):
    with np.load(os.path.join(GOLDEN, "lusolver.npz")) as z:
        return {k[len(name) + 1:]: z[k] for k in z.files if k.startswith(name + "_")
                and k[len(name) + 1:] in ("dim", "mode", "rows", "cols", "ops", "vals",
                                           "b", "x0", "x")}


def _oracle(g):
    mode, dim = int(g["mode"]), int(g["dim"])
    if mode == 2:
        return po.lu_block(dim, g["rows"], g["cols"], g["vals"], g["b"], g["x0"]), 5
    return po.lu_scalar(mode, dim, g["rows"], g["cols"], g["ops"], g["vals"], g["b"], g["x0"])


@pytest.mark.parametrize("name", NAMES)
def test_oracle_matches_reference_fixture(name):
    g = _case(name)
    x, it = _oracle(g)
    assert np.array_equal(x, g["x"])


def test_fixtures_cover_early_exit():
    its = [_oracle(_case(n))[1] for n in NAMES]
    assert min(its) < 5 and max(its) == 5


@pytest.mark.ref
@pytest.mark.parametrize("mode", [0, 1, 2])
@pytest.mark.parametrize("seed", [1, 2, 3])
def test_oracle_matches_reference_random(ref_available, mode, seed):
    import sys
    sys.path.insert(0, GOLDEN)
    from make_golden import lu_system
    from oracle import refrun
    dim, rows, cols, ops, vals, b, x0 = lu_system((9, 7), mode == 2, 5.0 + 20 * (seed == 3), seed)
    xr = refrun.run_lu(mode, dim, rows, cols, ops, vals, b, x0)
    g = dict(mode=np.array(mode), dim=np.array(dim), rows=rows, cols=cols, ops=ops, vals=vals,
             b=b, x0=x0)
    x, _ = _oracle(g)
    assert np.array_equal(x, xr)


@pytest.mark.gpu
@pytest.mark.parametrize("name", NAMES)
def test_gpu_matches_reference_fixture(name):
    from mstcfd.lusgs import SparseSystem
    g = _case(name)
    mode, dim = int(g["mode"]), int(g["dim"])
    s = SparseSystem(4 if mode == 2 else 1, dim, g["rows"], g["cols"], g["ops"], g["vals"])
    x, it = s.solve(g["b"], g["x0"], method=1 if mode == 1 else 0)
    assert np.array_equal(x, g["x"])
    assert it == _oracle(g)[1]
    f, b = s.levels()
    assert f > 1 and b > 1


@pytest.mark.gpu
@pytest.mark.parametrize("mode", [0, 1, 2])
def test_gpu_matches_oracle_large(mode):
    import sys
    sys.path.insert(0, GOLDEN)
    from make_golden import lu_system
    from mstcfd.lusgs import SparseSystem
    dim, rows, cols, ops, vals, b, x0 = lu_system((60, 40), mode == 2, 6.0, 77 + mode)
    g = dict(mode=np.array(mode), dim=np.array(dim), rows=rows, cols=cols, ops=ops, vals=vals,
             b=b, x0=x0)
    xo, ito = _oracle(g)
    s = SparseSystem(4 if mode == 2 else 1, dim, rows, cols, ops, vals)
    x, it = s.solve(b, x0, method=1 if mode == 1 else 0)
    assert np.array_equal(x, xo)
    assert it == ito


@pytest.mark.gpu
def test_gpu_rejects_bad_input():
    from mstcfd import MstError
    from mstcfd.lusgs import SparseSystem
    with pytest.raises(MstError):
        SparseSystem(1, 4, [0, 5], [0, 1], [0, 0], [1.0, 2.0])
    s = SparseSystem(4, 2, [0, 1], [0, 1], None, np.tile(np.eye(4).ravel(), 2))
    with pytest.raises(MstError):
        s.solve(np.ones(8), np.ones(8), method=1)
