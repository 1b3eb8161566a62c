"""CPU restatement of the learned initial-field network (numpy).

TEST INFRASTRUCTURE ONLY: the checker of the product's mst_mpnn_* entry
points (mst-cfd_gb300/csrc/mpnn.cu).  The reference has no learned part, so
this restates the project's own network and its backward pass:

  h0 = relu(We x + be)
  h_{l+1} = h_l + relu(Wl [h_l, mean_{j in N(c)} h_j] + bl),  l = 0..2
  y = Wd h3 + bd,  loss = mean((y - t)^2)

With ``bf16=True`` every GEMM operand is rounded to BF16 at the points the
GPU rounds it (weights, features, the [h, mean] concatenation, h3, dY, the
pre-activation gradients); accumulation in FP64 then FP32, the residual
stream FP32.  With ``bf16=False`` the same network in FP64, for finite-
difference checks of the backward pass itself.
"""
import numpy as np

W, IN, INK, OUT, LAYERS = 128, 16, 64, 4, 3
SHAPES = [(W, INK), (W,), (W, 2 * W), (W,), (W, 2 * W), (W,), (W, 2 * W), (W,), (OUT, W), (OUT,)]


def num_params():
    return int(sum(np.prod(s) for s in SHAPES))


def unpack(flat):
    out, o = [], 0
    for s in SHAPES:
        n = int(np.prod(s))
        out.append(np.asarray(flat[o:o + n]).reshape(s))
        o += n
    return out


def pack(ts):
    return np.concatenate([np.asarray(t, np.float64).ravel() for t in ts])


def bf16(x):
    """Round to the nearest BF16 (ties to even), returned as FP32."""
    u = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32)
    r = ((u >> 16) & 1) + 0x7FFF
    return (((u + r) >> 16) << 16).astype(np.uint32).view(np.float32)


class Net:
    def __init__(self, params, bf16_ops=True):
        self.p = [np.asarray(t, np.float64) for t in unpack(params)]
        self.b = bf16_ops

    def _r(self, x):
        return bf16(x).astype(np.float64) if self.b else np.asarray(x, np.float64)

    def _f(self, x):
        return np.asarray(x, np.float32).astype(np.float64) if self.b else x

    def forward(self, feats, ptr, nbr):
        p = self.p
        n = len(feats)
        x = np.zeros((n, INK))
        x[:, :IN] = feats
        x = self._r(x)
        deg = np.diff(ptr)
        owner = np.repeat(np.arange(n), deg)
        h = [self._f(np.maximum(x @ self._r(p[0]).T + p[1], 0.0))]
        z = []
        for l in range(LAYERS):
            hl = h[-1]
            agg = np.zeros_like(hl)
            np.add.at(agg, owner, hl[nbr])
            agg = agg / np.maximum(deg, 1)[:, None]
            zl = np.concatenate([self._r(hl), self._r(self._f(agg))], 1)
            z.append(zl)
            pre = self._f(zl @ self._r(p[2 + 2 * l]).T + p[3 + 2 * l])
            h.append(self._f(hl + np.maximum(pre, 0.0)))
        hb = self._r(h[-1])
        y = self._f(hb @ self._r(p[8]).T + p[9])
        self.cache = (x, h, z, hb, owner, deg, ptr, nbr)
        return y

    def backward(self, y, t):
        p = self.p
        x, h, z, hb, owner, deg, ptr, nbr = self.cache
        n = len(y)
        d = self._f(y - t)
        loss = float(np.mean(d * d))
        dy = self._f(2.0 * d / (n * OUT))
        g = [None] * len(p)
        dyb = self._r(dy)
        g[8] = dyb.T @ hb
        g[9] = dy.sum(0)
        dh = self._f(dyb @ self._r(p[8]))
        for l in reversed(range(LAYERS)):
            r = self._f(h[l + 1] - h[l])
            dp = np.where(r > 0, dh, 0.0)
            dpb = self._r(dp)
            g[2 + 2 * l] = dpb.T @ z[l]
            g[3 + 2 * l] = dp.sum(0)
            dz = self._f(dpb @ self._r(p[2 + 2 * l]))
            dh_new = dh + dz[:, :W]
            back = dz[owner, W:] / deg[owner][:, None]
            np.add.at(dh_new, nbr, back)
            dh = self._f(dh_new)
        dp = np.where(h[0] > 0, dh, 0.0)
        g[0] = self._r(dp).T @ x
        g[1] = dp.sum(0)
        return loss, g


def init_params(seed):
    """Glorot-uniform weights (first layer over its 16 real inputs), zero
    biases; a different generator from the product's, for tests that set
    the weights explicitly."""
    rng = np.random.default_rng(seed)
    out = []
    for i, s in enumerate(SHAPES):
        if len(s) == 1:
            out.append(np.zeros(s))
            continue
        fan_in = IN if i == 0 else s[1]
        a = np.sqrt(6.0 / (fan_in + s[0]))
        w = rng.uniform(-a, a, s)
        if i == 0:
            w[:, IN:] = 0.0
        out.append(w)
    return pack(out)
