"""The learned initial field (mst_mpnn_* of the C ABI): a message-passing
network over the cell adjacency whose dense layers run on the tensor cores
(BF16 operands, FP32 accumulation) for training and inference."""
import ctypes as C

import numpy as np

from . import capi

N_IN, N_OUT = 16, 4

_fp = C.POINTER(C.c_float)


def _f32(a, shape=None):
    a = np.ascontiguousarray(a, dtype=np.float32)
    if shape is not None and a.shape != shape:
        raise ValueError(f"expected shape {shape}, got {a.shape}")
    return a


class Network:
    def __init__(self, seed=0):
        L = capi.load()
        h = C.c_void_p()
        capi.check(L.mst_mpnn_create(C.c_uint64(seed), C.byref(h)))
        self._h = h
        self.n_params = L.mst_mpnn_num_params()
        self.n = 0

    def set_graph(self, features, nbr_ptr, nbr):
        f = _f32(features)
        n = f.shape[0]
        if f.shape != (n, N_IN):
            raise ValueError("features must be [n][16]")
        ptr = np.ascontiguousarray(nbr_ptr, dtype=np.int32)
        nb = np.ascontiguousarray(nbr, dtype=np.int32)
        if len(nb) == 0:
            nb = np.zeros(1, np.int32)
        capi.check(capi.load().mst_mpnn_set_graph(
            self._h, n, f.ctypes.data_as(_fp), ptr.ctypes.data_as(capi._ip),
            nb.ctypes.data_as(capi._ip)))
        self.n = n

    def set_targets(self, t):
        t = _f32(t, (self.n, N_OUT))
        capi.check(capi.load().mst_mpnn_set_targets(self._h, t.ctypes.data_as(_fp)))

    def forward(self):
        y = np.zeros((self.n, N_OUT), np.float32)
        capi.check(capi.load().mst_mpnn_forward(self._h, y.ctypes.data_as(_fp)))
        return y

    def backward(self):
        loss = C.c_double()
        capi.check(capi.load().mst_mpnn_backward(self._h, C.byref(loss)))
        return loss.value

    def params(self):
        out = np.zeros(self.n_params, np.float32)
        capi.check(capi.load().mst_mpnn_get(self._h, 0, out.ctypes.data_as(_fp)))
        return out

    def grads(self):
        out = np.zeros(self.n_params, np.float32)
        capi.check(capi.load().mst_mpnn_get(self._h, 1, out.ctypes.data_as(_fp)))
        return out

    def set_params(self, w):
        w = _f32(w, (self.n_params,))
        capi.check(capi.load().mst_mpnn_set_weights(self._h, w.ctypes.data_as(_fp)))

    def adam_step(self, lr):
        capi.check(capi.load().mst_mpnn_adam_step(self._h, C.c_float(lr)))

    def profile(self, on=True):
        """Start (or stop) timing every tensor-core GEMM launch with CUDA
        events; either clears what was recorded."""
        capi.check(capi.load().mst_mpnn_profile(self._h, 1 if on else 0))

    def profile_read(self):
        """Summed GEMM time (ms), 2MNK flops, operand/result bytes and
        launch count since the last profile()/profile_read(); clears them."""
        out = np.zeros(4)
        capi.check(capi.load().mst_mpnn_profile_read(self._h, out.ctypes.data_as(capi._dp)))
        return {"ms": float(out[0]), "flops": float(out[1]), "bytes": float(out[2]),
                "launches": int(out[3])}

    def close(self):
        h = getattr(self, "_h", None)
        if h:
            capi.load().mst_mpnn_destroy(h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
