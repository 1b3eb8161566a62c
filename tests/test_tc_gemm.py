"""The BF16 tensor-core GEMMs (tcgen05, TMEM accumulator) of the learned
initial field, against an FP32 numpy product of the same BF16 inputs:
FP32 accumulation, so agreement to a few ulps of FP32 times sqrt(K).  Shapes
with K <= 256 run the persistent TMA kernel (the large ones with several
row tiles per CTA, both accumulators and the copy ring wrapping; 4 outputs
in a 128-wide tile of which the copy fills the rest with zeros); split K
runs the split TMA kernel (one tile per CTA per chunk; 4 rows or 64
outputs with the rest of the tile filled with zeros); K above 256 and the
swapped-stride layout run the cp.async kernel (its 16-wide tile for 16
outputs or fewer)."""
import ctypes as C

import numpy as np
import pytest


def bf16_bits(x):
    """Round-to-nearest-even FP32 -> BF16 bit patterns."""
    u = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32)
    r = ((u >> 16) & 1) + 0x7FFF
    return ((u + r) >> 16).astype(np.uint16)


def bf16_value(bits):
    return (bits.astype(np.uint32) << 16).view(np.float32)


def test_bf16_rounding_helper():
    x = np.array([1.0, 1.00390625, 1.01171875, -3.14159, 65504.0], np.float32)
    v = bf16_value(bf16_bits(x))
    assert v[0] == 1.0 and v[1] == 1.0 and v[2] == 1.015625
    assert np.all(np.abs(v - x) <= np.abs(x) * 2.0 ** -8)


def _run(M, N, K, relu, bias, layout=0, seed=0):
    from mstcfd import capi
    rng = np.random.default_rng(seed)
    A = bf16_bits(rng.standard_normal((M, K)).astype(np.float32))
    B = bf16_bits(rng.standard_normal((N, K)).astype(np.float32))
    b = rng.standard_normal(N).astype(np.float32) if bias else None
    Cout = np.zeros((M, N), np.float32)
    st = capi.load().mst_tc_gemm_check(
        A.ctypes.data_as(C.POINTER(C.c_uint16)), B.ctypes.data_as(C.POINTER(C.c_uint16)),
        b.ctypes.data_as(C.POINTER(C.c_float)) if b is not None else None,
        Cout.ctypes.data_as(C.POINTER(C.c_float)), M, N, K, int(relu), int(layout))
    ref = bf16_value(A).astype(np.float64) @ bf16_value(B).astype(np.float64).T
    if b is not None:
        ref = ref + b
    if relu:
        ref = np.maximum(ref, 0)
    return st, Cout, ref


@pytest.mark.gpu
@pytest.mark.parametrize("M,N,K", [(128, 128, 64), (256, 128, 256), (384, 256, 128),
                                   (1000, 4, 128), (130, 128, 64), (89600, 256, 256),
                                   (40000, 128, 64), (1000, 48, 192), (1000, 4, 320),
                                   (256, 128, 512)])
@pytest.mark.parametrize("relu,bias", [(0, 0), (1, 1)])
def test_tc_gemm_matches_numpy(M, N, K, relu, bias):
    from mstcfd import capi
    st, got, ref = _run(M, N, K, relu, bias)
    assert st == capi.OK, capi.load().mst_last_error()
    tol = 1e-5 * np.sqrt(K) * (np.abs(ref).max() + 1)
    assert np.abs(got - ref).max() <= tol


@pytest.mark.gpu
@pytest.mark.parametrize("M,N,K,chunk", [(128, 256, 4096, 512), (4, 128, 2048, 192),
                                         (128, 64, 1280, 64)])
def test_tc_gemm_split_k(M, N, K, chunk):
    from mstcfd import capi
    st, got, ref = _run(M, N, K, 0, 0, layout=chunk, seed=2)
    assert st == capi.OK, capi.load().mst_last_error()
    tol = 1e-5 * np.sqrt(K) * (np.abs(ref).max() + 1)
    assert np.abs(got - ref).max() <= tol


@pytest.mark.gpu
@pytest.mark.parametrize("K", [64, 256])
def test_tc_gemm_wait_timeout_reports_and_recovers(K):
    """A bounded device wait that runs out: with the wait limit at 0 every
    mbarrier wait of the GEMM gives up at once, the kernel drains its own
    MMAs, frees its tensor memory and returns, and the call reports
    MST_ETIMEOUT; with the default limit back the next call is correct."""
    from mstcfd import capi
    L = capi.load()
    try:
        assert L.mst_set_wait_limit(0) == capi.OK
        st, _, _ = _run(256, 128, K, 0, 0)
        assert st == capi.ETIMEOUT
        assert b"timed out" in L.mst_last_error()
    finally:
        L.mst_set_wait_limit(-1)
    st, got, ref = _run(256, 128, K, 0, 0)
    assert st == capi.OK, L.mst_last_error()
    assert np.abs(got - ref).max() <= 1e-5 * np.sqrt(K) * (np.abs(ref).max() + 1)
