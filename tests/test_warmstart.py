"""Learned warm start of the batched steady solves (config 5 in small):
the network, trained on the GPU on ramps the batched solver converged
itself, gives initial fields from which the test ramps (disjoint seeds)
reach the same residual tolerance (the cold start's absolute target) in
fewer iterations than from free stream with the plain FP64 options, and
reach it with the production options too, converging to the same field up to the shock
profiles the frozen limiter selects (RMS difference below 1%)."""
import numpy as np
import pytest


@pytest.mark.gpu
def test_warm_start_beats_cold_start():
    from mstcfd import Mesh, batch, warmstart as ws
    from mstcfd import meshgen as mg
    from mstcfd.mpnn import Network

    def build(fam):
        out = []
        for p in fam:
            m, _ = ws.case_setup(p)
            mesh = Mesh.from_arrays(m["node_xy"], m["face_nodes"], m["face_cells"], m["zones"],
                                    m["n_cells"])
            out.append((p, m, mesh, batch.case_params(mg.freestream(p["mach"]))))
        return out

    kw = dict(flux=1, order=2, limiter=1, precision=1)
    # training ramps of the test ramps' own size range, disjoint seeds
    train = build(mg.wedge_family(24, cells=(5000, 8000), seed=4242))
    tb = batch.Batch([(mesh, cp) for _, _, mesh, cp in train], implicit=dict(max_iter=6000), **kw)
    tb.set_state([mg.freestream(p["mach"], mesh.n_cells) for p, _, mesh, _ in train])
    tb.solve()
    conv = tb.case_status()["conv_iter"]
    qs = tb.state()
    samples = []
    for k, (p, m, mesh, _) in enumerate(train):
        if conv[k] >= 0:
            ptr, nbr = ws.neighbours(m)
            samples.append((ws.features(m, mesh.arrays(), p), ptr, nbr,
                            ws.targets(qs[k], p["mach"])))
    assert len(samples) >= 18
    net = Network(seed=5)
    hist = ws.train(net, samples, steps=600, lr=2e-3, per_step=4)
    assert hist[-10:].mean() < 0.3 * hist[:10].mean()
    test = build(mg.wedge_family(4, cells=(5000, 8000), seed=9191))
    warm = []
    for p, m, mesh, _ in test:
        ptr, nbr = ws.neighbours(m)
        warm.append(ws.state(ws.predict(net, ws.features(m, mesh.arrays(), p), ptr, nbr),
                             p["mach"]))
    cold = [mg.freestream(p["mach"], mesh.n_cells) for p, _, mesh, _ in test]
    prod = dict(fp32_until=1e-5, sweep_fp32=1, fp32_window=1000)
    out = {}
    first = None
    for name, q0, opts in (("cold", cold, {}), ("warm", warm, {}),
                           ("cold_prod", cold, prod), ("warm_prod", warm, prod)):
        b = batch.Batch([(mesh, cp) for _, _, mesh, cp in test],
                        implicit=dict(max_iter=6000, **opts), **kw)
        b.set_state(q0)
        if name.startswith("warm"):
            b.set_l2_ref(first)  # the cold start's absolute residual target
        b.solve()
        st = b.case_status()
        if name == "cold":
            first = st["first_l2"]
        out[name] = (st["conv_iter"], b.state())
        b.close()
    cc, qc = out["cold"]
    cw, qw = out["warm"]
    assert np.all(cc >= 0) and np.all(cw >= 0)
    # what the network gains: fewer iterations to the same absolute
    # residual, per case (median) and over the batch (total)
    assert np.median(cw) < np.median(cc)
    assert cw.sum() < cc.sum(), (cw, cc)
    # with the production options (FP32 residual phase, FP32 sweeps; each
    # case leaves the FP32 phase on its own) the warm start reaches the
    # same tolerance too.  On ramps this small it does not take fewer
    # iterations (5,386 against 5,099 in total on these four): the gain in
    # wall time appears on the bench's batch of 20k-60k-cell ramps, through
    # its slowest cases
    cp_, qcp = out["cold_prod"]
    wp_, qwp = out["warm_prod"]
    assert np.all(cp_ >= 0) and np.all(wp_ >= 0)
    for a, c in zip(qwp, qcp):
        assert np.sqrt(np.mean((a - c) ** 2)) / np.sqrt(np.mean(c ** 2)) < 1e-2
    # both meet the tolerance; the fields differ only where the frozen
    # limiter (frozen at a different point of each run) picks a different
    # discrete shock profile
    for a, c in zip(qw, qc):
        rms = np.sqrt(np.mean((a - c) ** 2)) / np.sqrt(np.mean(c ** 2))
        assert rms < 1e-2, rms
    net.close()


def test_features_targets_and_union():
    from mstcfd import Mesh, warmstart as ws
    from mstcfd import meshgen as mg
    fam = mg.wedge_family(2, cells=(1500, 2500), seed=31)
    parts = []
    for p in fam:
        m = mg.wedge(p["cells"], p["angle"], seed=p["seed"])
        ptr, nbr = ws.neighbours(m)
        assert ptr[-1] == len(nbr) and np.all(np.diff(ptr) <= 3)
        q = mg.freestream(p["mach"], int(m["n_cells"]))
        q[:, 0] *= 1.3
        t = ws.targets(q, p["mach"])
        assert np.allclose(ws.state(t, p["mach"]), q, rtol=1e-5, atol=1e-6)
        parts.append((np.zeros((int(m["n_cells"]), 16), np.float32), ptr, nbr, t))
    f, ptr, nbr, t = ws.union(parts)
    n0 = len(parts[0][0])
    assert len(f) == len(t) == n0 + len(parts[1][0])
    assert ptr[-1] == len(nbr) and ptr[n0] == parts[0][1][-1]
    assert nbr[ptr[n0]:].min() >= n0 and nbr[:ptr[n0]].max() < n0
