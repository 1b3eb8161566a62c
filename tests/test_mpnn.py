"""The learned initial-field network.

* oracle: its FP64 backward pass against central finite differences;
* GPU (through the C ABI, tensor-core forward and backward): outputs, loss
  and every parameter gradient against the oracle with the GPU's BF16
  rounding points, on a mesh graph; Adam training lowers the loss.
"""
import numpy as np
import pytest

from oracle import mpnn_ref as mr


def _graph(n_cells=600, seed=0):
    """Cell adjacency of a small triangle mesh and random features/targets."""
    from mstcfd import meshgen as mg
    m = mg.tri_box(16, 10, 2.0, 1.0, jitter=0.2, seed=seed)
    fc = m["face_cells"]
    fc = fc[fc[:, 1] >= 0]
    n = int(m["n_cells"])
    a = np.concatenate([fc[:, 0], fc[:, 1]])
    b = np.concatenate([fc[:, 1], fc[:, 0]])
    order = np.lexsort((b, a))
    a, b = a[order], b[order]
    ptr = np.zeros(n + 1, np.int32)
    np.add.at(ptr, a + 1, 1)
    ptr = np.cumsum(ptr).astype(np.int32)
    rng = np.random.default_rng(seed + 1)
    feats = rng.standard_normal((n, mr.IN)).astype(np.float32)
    targ = (0.3 * rng.standard_normal((n, mr.OUT))).astype(np.float32)
    return feats, ptr, b.astype(np.int32), targ


def test_oracle_backward_matches_finite_differences():
    feats, ptr, nbr, targ = _graph(seed=2)
    feats, targ = feats[:40], targ[:40]
    # keep the graph closed over the first 40 cells
    keep = np.arange(40)
    sub_ptr, sub_nbr = [0], []
    for c in keep:
        nb = [j for j in nbr[ptr[c]:ptr[c + 1]] if j < 40]
        sub_nbr += nb
        sub_ptr.append(len(sub_nbr))
    ptr, nbr = np.array(sub_ptr), np.array(sub_nbr, int)
    w = mr.init_params(3)
    rng = np.random.default_rng(4)
    p = mr.unpack(w)
    for i in (1, 3, 5, 7, 9):  # nonzero biases
        p[i] = 0.1 * rng.standard_normal(p[i].shape)
    w = mr.pack(p)
    net = mr.Net(w, bf16_ops=False)
    y = net.forward(feats, ptr, nbr)
    _, g = net.backward(y, targ)
    gflat = mr.pack(g)
    idx = rng.choice(len(w), 40, replace=False)
    idx = idx[np.abs(gflat[idx]) > 0] if np.any(np.abs(gflat[idx]) > 0) else idx
    for k in idx[:25]:
        e = 1e-6
        wp, wm = w.copy(), w.copy()
        wp[k] += e
        wm[k] -= e
        lp = np.mean((mr.Net(wp, False).forward(feats, ptr, nbr) - targ) ** 2)
        lm = np.mean((mr.Net(wm, False).forward(feats, ptr, nbr) - targ) ** 2)
        fd = (lp - lm) / (2 * e)
        assert abs(fd - gflat[k]) <= 1e-6 + 1e-4 * abs(fd), (k, fd, gflat[k])


def _rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30)


@pytest.mark.gpu
def test_gpu_forward_backward_match_oracle():
    from mstcfd.mpnn import Network
    feats, ptr, nbr, targ = _graph(seed=5)
    w = mr.init_params(7)
    p = mr.unpack(w)
    rng = np.random.default_rng(8)
    for i in (1, 3, 5, 7, 9):
        p[i] = 0.1 * rng.standard_normal(p[i].shape)
    w = mr.pack(p).astype(np.float32)
    net = Network(seed=1)
    net.set_params(w)
    net.set_graph(feats, ptr, nbr)
    net.set_targets(targ)
    y = net.forward()
    loss = net.backward()
    g = net.grads()
    ref = mr.Net(w.astype(np.float64), bf16_ops=True)
    yr = ref.forward(feats.astype(np.float64), ptr, nbr)
    lr_, gr = ref.backward(yr, targ.astype(np.float64))
    assert _rel(y, yr) < 2e-3
    assert abs(loss - lr_) <= 1e-3 * lr_
    gg = mr.unpack(g)
    for i, (a, b) in enumerate(zip(gg, gr)):
        assert _rel(a, b) < 2e-2, (i, _rel(a, b))
    net.close()


@pytest.mark.gpu
def test_gpu_adam_training_lowers_the_loss():
    from mstcfd.mpnn import Network
    feats, ptr, nbr, _ = _graph(seed=9)
    # a smooth target the network can fit: functions of the features
    targ = np.stack([np.tanh(feats[:, 0]), 0.5 * feats[:, 1], np.sin(feats[:, 2]),
                     0.2 * feats[:, 3] * feats[:, 4]], 1).astype(np.float32)
    net = Network(seed=3)
    net.set_graph(feats, ptr, nbr)
    net.set_targets(targ)
    losses = []
    for _ in range(200):
        net.forward()
        losses.append(net.backward())
        net.adam_step(2e-3)
    assert np.all(np.isfinite(losses))
    assert losses[-1] < 0.2 * losses[0]
    net.close()


@pytest.mark.gpu
def test_gpu_gemm_profile_counts_the_launches():
    """Live GEMM timing: a forward runs 5 tensor-core GEMMs (encoder, three
    layers, decoder) whose 2MNK flops are known; a backward adds 9 (a weight
    gradient and an input gradient per layer, the decoder's two, the
    encoder's weight gradient)."""
    from mstcfd.mpnn import Network
    feats, ptr, nbr, targ = _graph(seed=4)
    n = len(feats)
    np_ = (n + 127) // 128 * 128
    nk = (n + 63) // 64 * 64
    net = Network(seed=1)
    net.set_graph(feats, ptr, nbr)
    net.set_targets(targ)
    net.profile(True)
    net.forward()
    g = net.profile_read()
    w, z, ink, out = 128, 256, 64, 4
    assert g["launches"] == 5
    assert g["flops"] == 2.0 * np_ * (w * ink + 3 * w * z + out * w)
    assert g["ms"] > 0 and g["bytes"] > 0
    net.backward()
    g = net.profile_read()
    assert g["launches"] == 9
    wgrad = 2.0 * nk * (out * w + 3 * w * z + w * ink)
    dgrad = 2.0 * np_ * (w * ink + 3 * z * w)
    assert g["flops"] == wgrad + dgrad
    net.profile(False)
    net.forward()
    assert net.profile_read()["launches"] == 0
    net.close()
