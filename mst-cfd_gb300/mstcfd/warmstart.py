"""Learned warm start of the batched steady solves.

The network (mstcfd.mpnn, trained and run on the tensor cores) maps per-cell
geometry and the case's flow parameters to the converged field of the
compression-ramp family (meshgen.wedge):

  features (16 per cell): centroid (x/3, y/1.5); the unit outward normals of
    the cell's first three faces; distance to the nearest wall face; height
    above the floor as a fraction of the channel; a flag for cells past the
    ramp corner; sqrt(V) / h of the mesh; (Mach - 2.25) / 0.75,
    (angle - 10) / 5, (log10 Re - 3.5) / 0.5; 0
  outputs (4 per cell): log(rho / rho_inf), u / U_inf - 1, v / U_inf,
    log(p / p_inf)  (positive density and pressure by construction)

Training pairs come from cases the batched solver itself converged (cold
start); a warm-started case counts only when it reaches the same residual
tolerance as the cold start, and its final field is compared to the cold
start's.
"""
import numpy as np

from . import meshgen as mg

GAMMA = 1.4
CV = 1.0 / (GAMMA * (GAMMA - 1.0))


def case_params_of(p):
    """Batch case parameters of one family member (free stream, laminar
    transport coefficients of its Reynolds number)."""
    from . import batch
    mu = p["mach"] / p["reynolds"]
    return batch.case_params(mg.freestream(p["mach"]), mu=mu, lambda_=-2.0 / 3.0 * mu,
                             kappa=mu * GAMMA * CV / 0.72, cv=CV)


def case_setup(p):
    """Mesh dict and batch case parameters of one family member."""
    return mg.wedge(p["cells"], p["angle"], seed=p["seed"]), case_params_of(p)


def neighbours(m):
    """CSR lists of interior-face neighbours (file cell order)."""
    fc = np.asarray(m["face_cells"])
    fc = fc[fc[:, 1] >= 0]
    n = int(m["n_cells"])
    a = np.concatenate([fc[:, 0], fc[:, 1]])
    b = np.concatenate([fc[:, 1], fc[:, 0]])
    o = np.lexsort((b, a))
    a, b = a[o], b[o]
    ptr = np.zeros(n + 1, np.int64)
    np.add.at(ptr, a + 1, 1)
    return np.cumsum(ptr).astype(np.int32), b.astype(np.int32)


def features(m, arrays, p, length=3.0, height=1.5, ramp_x=0.5):
    """[n_cells][16] float32 features of one case (see the module doc)."""
    from scipy.spatial import cKDTree
    n = int(m["n_cells"])
    ctr = arrays["cell_ctr"]
    f = np.zeros((n, 16), np.float32)
    f[:, 0] = ctr[:, 0] / length
    f[:, 1] = ctr[:, 1] / height
    ptr, dof = arrays["cell_ptr"], arrays["cell_dof"]
    for k in range(3):
        idx = np.minimum(ptr[:-1] + k, ptr[1:] - 1)
        d = dof[idx]
        nrm = np.linalg.norm(d, axis=1)[:, None]
        f[:, 2 + 2 * k:4 + 2 * k] = np.where(nrm > 0, d / np.maximum(nrm, 1e-300), 0.0)
    # wall faces: zone type 3
    ftype = np.zeros(len(m["face_cells"]), np.int32)
    for _, first, last, ty in m["zones"]:
        ftype[first - 1:last] = ty
    fctr = arrays["face_ctr"]
    walls = fctr[ftype == mg.WALL]
    if len(walls):
        dist, _ = cKDTree(walls).query(ctr)
    else:
        dist = np.full(n, height)
    f[:, 8] = dist / height
    yw = np.maximum(0.0, ctr[:, 0] - ramp_x) * np.tan(np.radians(p["angle"]))
    f[:, 9] = (ctr[:, 1] - yw) / (height - yw)
    f[:, 10] = (ctr[:, 0] > ramp_x).astype(np.float32)
    h = np.sqrt(length * height / n)
    f[:, 11] = np.sqrt(arrays["cell_vol"]) / h
    f[:, 12] = (p["mach"] - 2.25) / 0.75
    f[:, 13] = (p["angle"] - 10.0) / 5.0
    f[:, 14] = (np.log10(p["reynolds"]) - 3.5) / 0.5
    return f


def targets(q, mach):
    """Network outputs of conserved states q [n][4] (free stream rho = 1,
    speed of sound 1)."""
    rho = q[:, 0]
    u, v = q[:, 1] / rho, q[:, 2] / rho
    p = (GAMMA - 1.0) * (q[:, 3] - 0.5 * rho * (u * u + v * v))
    return np.stack([np.log(rho), u / mach - 1.0, v / mach,
                     np.log(np.maximum(p, 1e-12) * GAMMA)], 1).astype(np.float32)


def state(y, mach):
    """Conserved states from network outputs."""
    y = np.asarray(y, np.float64)
    rho = np.exp(y[:, 0])
    u = mach * (1.0 + y[:, 1])
    v = mach * y[:, 2]
    p = np.exp(y[:, 3]) / GAMMA
    return mg.primitive_to_q(rho, u, v, p)


def union(parts):
    """One graph of several cases: (features, nbr_ptr, nbr, targets|None)."""
    feats, ptrs, nbrs, targs = [], [np.zeros(1, np.int64)], [], []
    cells = edges = 0
    for f, ptr, nbr, t in parts:
        feats.append(f)
        ptrs.append(np.asarray(ptr[1:], np.int64) + edges)
        nbrs.append(np.asarray(nbr, np.int64) + cells)
        if t is not None:
            targs.append(t)
        cells += len(f)
        edges += int(ptr[-1])
    return (np.concatenate(feats), np.concatenate(ptrs).astype(np.int32),
            np.concatenate(nbrs).astype(np.int32),
            np.concatenate(targs) if targs else None)


def train(net, samples, steps=400, lr=2e-3, per_step=4, seed=0, log=None):
    """Adam on random groups of `per_step` training cases; samples are
    (features, nbr_ptr, nbr, targets) per case.  Returns the loss history."""
    rng = np.random.default_rng(seed)
    hist = []
    for it in range(steps):
        pick = rng.choice(len(samples), size=min(per_step, len(samples)), replace=False)
        f, ptr, nbr, t = union([samples[i] for i in pick])
        net.set_graph(f, ptr, nbr)
        net.set_targets(t)
        net.forward()
        hist.append(net.backward())
        # cosine decay to a tenth
        net.adam_step(lr * (0.55 + 0.45 * np.cos(np.pi * it / steps)))
        if log and it % 50 == 0:
            log(it, hist[-1])
    return np.array(hist)


def predict(net, f, ptr, nbr):
    net.set_graph(f, ptr, nbr)
    return net.forward()
