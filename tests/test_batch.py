"""Batched steady solves (implicit LU-SGS over colour groups).

* oracle: the greedy colouring is a proper colouring; LU-SGS on an inviscid
  compression ramp converges to round-off and gives the oblique-shock
  density ratio of the theta-beta-Mach relation;
* GPU (through the C ABI): per case bit-identical to the oracle's
  iterations (FP64-exact, constant CFL), inviscid and viscous, for a batch
  of cases of different sizes and inflow states; colours equal the
  oracle's; mst_batch_solve (CUDA graph) reaches the tolerance and
  repeats bit-for-bit the plain iterations; the FP64 production path and
  the FP32 residual agree with the exact path to their rounding.
"""
import numpy as np
import pytest

from oracle import pyoracle as po

GAMMA = 1.4
CV = 1.0 / (GAMMA * (GAMMA - 1.0))


def _wedge(cells, angle, seed):
    from mstcfd import meshgen as mg
    return mg.wedge(cells, angle, seed=seed)


def _oracle_mesh(m):
    return po.mesh_from_arrays(m["node_xy"], m["face_nodes"], m["face_cells"], m["zones"],
                               m["n_cells"])


def _visc(mach, re):
    mu = mach / re
    return mu, -2.0 / 3.0 * mu, mu * GAMMA * CV / 0.72


def test_oracle_colors_are_proper():
    m = _wedge(3000, 12.0, 4)
    om = _oracle_mesh(m)
    col, n = po.greedy_colors(om)
    assert 2 <= n <= 4
    fc = om.face_cells[om.face_cells[:, 1] >= 0]
    assert np.all(col[fc[:, 0]] != col[fc[:, 1]])


def _beta(mach, theta):
    """Weak oblique-shock angle of the theta-beta-Mach relation."""
    from scipy.optimize import brentq
    t = np.radians(theta)
    f = lambda b: (2 / np.tan(b) * (mach ** 2 * np.sin(b) ** 2 - 1)
                   / (mach ** 2 * (GAMMA + np.cos(2 * b)) + 2)) - np.tan(t)
    mu = np.arcsin(1 / mach)
    return brentq(f, mu + 1e-6, np.radians(64.0))


def test_oracle_lusgs_inviscid_ramp_converges_to_oblique_shock():
    from mstcfd import meshgen as mg
    mach, theta = 2.0, 10.0
    m = _wedge(3000, theta, 1)
    om = _oracle_mesh(m)
    prm = po.params_ext(1, 2, limiter=1, quirks=0, inlet_q=mg.freestream(mach))
    col, _ = po.greedy_colors(om)
    q, hist = po.lusgs_iterate(om, prm, mg.freestream(mach, om.n_cells), col, 700,
                               cfl0=50.0, cfl_max=5000.0, omega=1.2)
    assert hist[-1] / hist[0] < 1e-10
    b = _beta(mach, theta)
    mn = mach * np.sin(b)
    ratio = (GAMMA + 1) * mn ** 2 / ((GAMMA - 1) * mn ** 2 + 2)
    # cells well behind the shock and away from the outlet corner
    x, y = om.cell_ctr[:, 0], om.cell_ctr[:, 1]
    xr = 0.5
    yw = (x - xr) * np.tan(np.radians(theta))
    ys = (x - xr) * np.tan(b)
    sel = (x > 1.2) & (x < 2.2) & (y > yw + 0.05) & (y < yw + 0.5 * (ys - yw))
    assert sel.sum() > 20
    assert abs(np.median(q[sel, 0]) - ratio) < 0.02 * ratio


# ---------------------------------------------------------------------------
# GPU
# ---------------------------------------------------------------------------
SPECS = [(1500, 8.0, 1.8, 3), (2600, 12.0, 2.4, 5), (2000, 6.0, 2.9, 7)]


def _batch_cases(viscous, specs=SPECS):
    from mstcfd import Mesh, batch
    from mstcfd import meshgen as mg
    out = []
    for cells, angle, mach, seed in specs:
        m = _wedge(cells, angle, seed)
        mesh = Mesh.from_arrays(m["node_xy"], m["face_nodes"], m["face_cells"], m["zones"],
                                m["n_cells"])
        mu, lam, kap = _visc(mach, 2000.0 + 1000 * seed) if viscous else (0.0, 0.0, 0.0)
        out.append((m, mesh, mach,
                    batch.case_params(mg.freestream(mach), mu=mu, lambda_=lam, kappa=kap, cv=CV)))
    return out


SPECS_STALL = [(1500, 8.0, 1.8, 3), (2600, 12.0, 2.4, 5), (2000, 6.0, 2.9, 7)]


@pytest.mark.parametrize("freeze", [0.0, 1e-2])
def test_oracle_limiter_freezing_removes_the_stall(freeze):
    """Minmod's switching stalls LU-SGS on two of these ramps; with the
    limiter frozen at 1e-2 every case reaches 1e-8."""
    from mstcfd import meshgen as mg
    conv = []
    for cells, angle, mach, seed in SPECS_STALL:
        om = _oracle_mesh(_wedge(cells, angle, seed))
        prm = po.params_ext(1, 2, limiter=1, quirks=0, inlet_q=mg.freestream(mach))
        col, _ = po.greedy_colors(om)
        _, h = po.lusgs_iterate(om, prm, mg.freestream(mach, om.n_cells), col, 1000,
                                cfl0=50.0, cfl_max=1000.0, omega=1.2, freeze_tol=freeze,
                                tol=1e-8)
        conv.append(h[-1] / h[0] < 1e-8)
    if freeze:
        assert all(conv)
    else:
        assert not all(conv)


@pytest.mark.gpu
@pytest.mark.parametrize("freeze,p_floor", [(0.0, 0.0), (0.9, 0.0), (0.0, 0.75)],
                         ids=["live", "frozen", "floor"])
@pytest.mark.parametrize("viscous", [0, 1], ids=["euler", "laminar"])
def test_gpu_batch_matches_oracle(viscous, freeze, p_floor):
    """A few iterations bit-identical to the restatement; the 'floor' case
    sets the temperature floor above the free stream's p / rho = 1/1.4, so
    it acts on every cell of every update."""
    from mstcfd import batch
    from mstcfd import meshgen as mg
    cases = _batch_cases(viscous)
    b = batch.Batch([(mesh, cp) for _, mesh, _, cp in cases],
                    implicit=dict(cfl0=40.0, cfl_max=40.0, omega=1.2, autotune=0,
                                  graph_iters=0, freeze_tol=freeze, p_floor=p_floor),
                    flux=1, order=2, limiter=1, precision=0, viscous=viscous)
    q0 = [mg.freestream(mach, mesh.n_cells) for _, mesh, mach, _ in cases]
    n_it = 70 if freeze else 12  # the freezing check runs every 50 iterations
    b.set_state(q0)
    b.iterate(n_it)
    got = b.state()
    cols = b.colors()
    st = b.case_status()
    for k, (m, mesh, mach, cp) in enumerate(cases):
        om = _oracle_mesh(m)
        col, _ = po.greedy_colors(om)
        assert np.array_equal(cols[k], col)
        prm = po.params_ext(1, 2, limiter=1, quirks=0, inlet_q=cp["inlet_q"], viscous=viscous,
                            mu=cp["mu"], lam=cp["lambda_"], kappa=cp["kappa"], cv=cp["cv"])
        q, hist = po.lusgs_iterate(om, prm, q0[k], col, n_it, cfl0=40.0, cfl_max=40.0,
                                   omega=1.2, freeze_tol=freeze, p_floor=p_floor)
        assert np.array_equal(got[k], q), k
        assert np.isclose(st["first_l2"][k], hist[0], rtol=1e-12)
        assert np.isclose(st["last_l2"][k], hist[-1], rtol=1e-12)
    b.close()


@pytest.mark.gpu
def test_gpu_batch_solve_converges_and_graph_is_deterministic():
    from mstcfd import batch
    from mstcfd import meshgen as mg
    cases = _batch_cases(0)
    kw = dict(flux=1, order=2, limiter=1, precision=1)
    imp = dict(cfl0=50.0, cfl_max=1000.0, omega=1.2, tol=1e-8, freeze_tol=1e-2, max_iter=3000)
    b = batch.Batch([(mesh, cp) for _, mesh, _, cp in cases],
                    implicit=dict(imp, graph_iters=10), **kw)
    q0 = [mg.freestream(mach, mesh.n_cells) for _, mesh, mach, _ in cases]
    b.set_state(q0)
    r = b.solve()
    assert r["n_converged"] == len(cases)
    st = b.case_status()
    assert np.all(st["conv_iter"] > 0)
    assert np.all(st["last_l2"] <= 1e-8 * st["first_l2"] * 1.0001)
    info = b.info()
    assert info["graph_iters"] == 10 and info["sweep_threads"] in (64, 128, 256)
    # the same number of plain iterations repeats the graph's result exactly
    b2 = batch.Batch([(mesh, cp) for _, mesh, _, cp in cases],
                     implicit=dict(imp, graph_iters=0, autotune=0), **kw)
    b2.set_state(q0)
    b2.iterate(r["iterations"])
    for a, c in zip(b.state(), b2.state()):
        assert np.array_equal(a, c)
    b.close()
    b2.close()


@pytest.mark.gpu
def test_gpu_batch_retires_diverged_cases():
    """Per-case divergence detection: two cases whose initial state is
    poisoned on the host (a NaN cell; a cell of negative pressure) are
    retired as MST_CASE_DIVERGED at their first iteration and cost nothing
    afterwards, while the healthy cases converge to exactly the states of
    the same batch without the poisoned ones."""
    from mstcfd import batch, capi
    from mstcfd import meshgen as mg
    cases = _batch_cases(0)
    kw = dict(flux=1, order=2, limiter=1, precision=1)
    imp = dict(cfl0=50.0, cfl_max=1000.0, omega=1.2, tol=1e-8, freeze_tol=1e-1, max_iter=3000,
               graph_iters=10)
    q0 = [mg.freestream(mach, mesh.n_cells) for _, mesh, mach, _ in cases]
    bad_nan = q0[0].copy()
    bad_nan[len(bad_nan) // 2, 0] = np.nan
    bad_p = q0[1].copy()
    bad_p[7, 3] = 0.25 * (bad_p[7, 1] ** 2 + bad_p[7, 2] ** 2) / bad_p[7, 0]  # E < kinetic
    poisoned = [(cases[0][1], cases[0][3]), (cases[1][1], cases[1][3])]
    all_cases = poisoned + [(mesh, cp) for _, mesh, _, cp in cases]
    b = batch.Batch(all_cases, implicit=imp, **kw)
    b.set_state([bad_nan, bad_p] + q0)
    r = b.solve()
    st = b.case_status()
    assert list(st["conv_iter"][:2]) == [capi.CASE_DIVERGED] * 2
    assert r["n_diverged"] == 2 and r["n_converged"] == len(cases)
    assert np.all(st["conv_iter"][2:] > 0)
    got = b.state()[2:]
    b.close()
    ref = batch.Batch([(mesh, cp) for _, mesh, _, cp in cases], implicit=imp, **kw)
    ref.set_state(q0)
    r2 = ref.solve()
    assert r2["iterations"] == r["iterations"] and r2["n_diverged"] == 0
    for a, c in zip(got, ref.state()):
        assert np.array_equal(a, c)
    ref.close()


@pytest.mark.gpu
def test_gpu_batch_solve_matches_oracle_solve():
    """FP64-exact batch solved to 1e-8 with limiter freezing: every case's
    final state and convergence iteration equal the oracle's single-case
    run (converged cases keep their state, so the batch composition does
    not matter)."""
    from mstcfd import batch
    from mstcfd import meshgen as mg
    cases = _batch_cases(0)
    imp = dict(cfl0=50.0, cfl_max=50.0, omega=1.2, tol=1e-8, freeze_tol=1e-2, max_iter=2000)
    b = batch.Batch([(mesh, cp) for _, mesh, _, cp in cases], implicit=dict(imp, graph_iters=10),
                    flux=1, order=2, limiter=1, precision=0)
    q0 = [mg.freestream(mach, mesh.n_cells) for _, mesh, mach, _ in cases]
    b.set_state(q0)
    r = b.solve()
    st = b.case_status()
    got = b.state()
    for k, (m, mesh, mach, cp) in enumerate(cases):
        om = _oracle_mesh(m)
        col, _ = po.greedy_colors(om)
        prm = po.params_ext(1, 2, limiter=1, quirks=0, inlet_q=cp["inlet_q"])
        q, hist = po.lusgs_iterate(om, prm, q0[k], col, r["iterations"], cfl0=50.0,
                                   cfl_max=50.0, omega=1.2, freeze_tol=1e-2, tol=1e-8)
        assert np.array_equal(got[k], q), k
        conv = np.nonzero(hist <= 1e-8 * hist[0])[0]
        assert len(conv) and st["conv_iter"][k] == conv[0]
    b.close()


@pytest.mark.gpu
@pytest.mark.parametrize("prec", [1, 2], ids=["fp64", "fp32"])
def test_gpu_batch_production_precisions_track_exact(prec):
    from mstcfd import batch
    from mstcfd import meshgen as mg
    cases = _batch_cases(0)
    q0 = [mg.freestream(mach, mesh.n_cells) for _, mesh, mach, _ in cases]
    out = {}
    for p in (0, prec):
        b = batch.Batch([(mesh, cp) for _, mesh, _, cp in cases],
                        implicit=dict(cfl0=40.0, cfl_max=40.0, omega=1.2, autotune=0,
                                      graph_iters=0, freeze_tol=0.0),
                        flux=1, order=2, limiter=1, precision=p)
        b.set_state(q0)
        b.iterate(30)
        out[p] = b.state()
        b.close()
    tol = 1e-9 if prec == 1 else 2e-4
    for a, c in zip(out[0], out[prec]):
        assert np.abs(a - c).max() <= tol * np.abs(a).max()


@pytest.mark.gpu
def test_gpu_batch_mixed_precision_reaches_tolerance():
    """FP32 residual until 1e-3, then FP64: every case reaches 1e-8 and the
    converged fields agree with the FP64-only solve."""
    from mstcfd import batch
    from mstcfd import meshgen as mg
    cases = _batch_cases(0)
    q0 = [mg.freestream(mach, mesh.n_cells) for _, mesh, mach, _ in cases]
    out = {}
    for fp32 in (0.0, 1e-3):
        b = batch.Batch([(mesh, cp) for _, mesh, _, cp in cases],
                        implicit=dict(fp32_until=fp32, max_iter=4000),
                        flux=1, order=2, limiter=1, precision=1)
        b.set_state(q0)
        r = b.solve()
        assert r["n_converged"] == len(cases), fp32
        out[fp32] = b.state()
        b.close()
    for a, c in zip(out[0.0], out[1e-3]):
        rms = np.sqrt(np.mean((a - c) ** 2)) / np.sqrt(np.mean(a ** 2))
        assert rms < 1e-3


@pytest.mark.gpu
def test_gpu_batch_mixed_phases_are_per_case():
    """Each case leaves the FP32-residual phase on its own: solved in a
    batch beside cases in either phase, a case ends bit-identical to the
    same case solved alone with the same options (constant CFL), at the
    same iteration -- a batch-wide switch would keep the early cases in
    FP32 until the last one is ready."""
    from mstcfd import batch
    from mstcfd import meshgen as mg
    cases = _batch_cases(0)
    imp = dict(cfl0=50.0, cfl_max=50.0, tol=1e-8, freeze_tol=1e-2, fp32_until=1e-3,
               fp32_window=100, max_iter=3000)
    kw = dict(flux=1, order=2, limiter=1, precision=1)
    q0 = [mg.freestream(mach, mesh.n_cells) for _, mesh, mach, _ in cases]
    b = batch.Batch([(mesh, cp) for _, mesh, _, cp in cases], implicit=imp, **kw)
    b.set_state(q0)
    r = b.solve()
    assert r["n_converged"] == len(cases)
    got, conv = b.state(), b.case_status()["conv_iter"]
    b.close()
    for k, (_, mesh, _, cp) in enumerate(cases):
        one = batch.Batch([(mesh, cp)], implicit=imp, **kw)
        one.set_state([q0[k]])
        one.solve()
        assert np.array_equal(one.state()[0], got[k]), k
        assert one.case_status()["conv_iter"][0] == conv[k], k
        one.close()


@pytest.mark.gpu
@pytest.mark.parametrize("fp32", [0.0, 1e-3], ids=["fp64", "mixed"])
def test_gpu_batch_restart_from_fallback_is_a_cold_start(fp32):
    """A case restarted from its fallback state iterates exactly as a solve
    started from it: case 1 starts from a perturbed state, restarts from
    the free stream after 40 iterations, and ends bit-identical to the
    cold start's case 1, 40 iterations later; the other cases are
    untouched."""
    from mstcfd import batch
    from mstcfd import meshgen as mg
    cases = _batch_cases(0)
    imp = dict(tol=1e-8, freeze_tol=0.1, fp32_until=fp32, fp32_window=100, max_iter=4000)
    kw = dict(flux=1, order=2, limiter=1, precision=1)
    q0 = [mg.freestream(mach, mesh.n_cells) for _, mesh, mach, _ in cases]
    cold = batch.Batch([(mesh, cp) for _, mesh, _, cp in cases], implicit=imp, **kw)
    cold.set_state(q0)
    cold.solve()
    qc, cc = cold.state(), cold.case_status()["conv_iter"]
    cold.close()
    assert np.all(cc >= 0)
    bad = [q.copy() for q in q0]
    bad[1] = bad[1] * np.array([1.1, 0.9, 1.0, 1.05])
    b = batch.Batch([(mesh, cp) for _, mesh, _, cp in cases], implicit=imp, **kw)
    b.set_state(bad)
    b.set_fallback(q0)
    b.iterate(40)
    b.restart([1])
    r = b.solve()
    st, qb = b.case_status(), b.state()
    b.close()
    assert r["n_restarted"] == 1 and list(st["restart_iter"]) == [-1, 40, -1]
    assert st["conv_iter"][1] == cc[1] + 40
    for k in range(len(cases)):
        assert np.array_equal(qb[k], qc[k]), k


@pytest.mark.gpu
def test_gpu_batch_restart_after_an_iteration_budget():
    """restart_after: every case not converged 40 iterations after the
    state was set restarts from its fallback state at the next graph
    launch boundary, once, and then iterates as a cold start would (final
    states bit-identical, convergence 40 iterations later)."""
    from mstcfd import batch
    from mstcfd import meshgen as mg
    cases = _batch_cases(0)
    imp = dict(tol=1e-8, freeze_tol=0.1, max_iter=4000, graph_iters=20)
    kw = dict(flux=1, order=2, limiter=1, precision=1)
    q0 = [mg.freestream(mach, mesh.n_cells) for _, mesh, mach, _ in cases]
    cold = batch.Batch([(mesh, cp) for _, mesh, _, cp in cases], implicit=imp, **kw)
    cold.set_state(q0)
    cold.solve()
    qc, cc = cold.state(), cold.case_status()["conv_iter"]
    cold.close()
    bad = [q * np.array([1.1, 0.9, 1.0, 1.05]) for q in q0]
    b = batch.Batch([(mesh, cp) for _, mesh, _, cp in cases],
                    implicit=dict(imp, restart_after=40), **kw)
    b.set_state(bad)
    b.set_fallback(q0)
    r = b.solve()
    st, qb = b.case_status(), b.state()
    b.close()
    assert r["n_restarted"] == len(cases) and np.all(st["restart_iter"] == 40)
    assert np.array_equal(st["conv_iter"], cc + 40)
    for k in range(len(cases)):
        assert np.array_equal(qb[k], qc[k]), k


@pytest.mark.gpu
def test_gpu_batch_restart_when_projected_past_the_cap():
    """restart_projected: with a tolerance no case can reach in 400
    iterations (1e-30), every case projects past the cap in the windows
    ending at iterations 80 and 120 and restarts from its fallback state at
    120; at the cap its state equals a cold start's after 280 iterations,
    bit for bit."""
    from mstcfd import batch
    from mstcfd import meshgen as mg
    cases = _batch_cases(0)
    imp = dict(tol=1e-30, freeze_tol=0.1, graph_iters=20)
    kw = dict(flux=1, order=2, limiter=1, precision=1)
    q0 = [mg.freestream(mach, mesh.n_cells) for _, mesh, mach, _ in cases]
    cold = batch.Batch([(mesh, cp) for _, mesh, _, cp in cases], implicit=dict(imp, max_iter=280),
                       **kw)
    cold.set_state(q0)
    cold.solve()
    qc = cold.state()
    cold.close()
    bad = [q * np.array([1.1, 0.9, 1.0, 1.05]) for q in q0]
    b = batch.Batch([(mesh, cp) for _, mesh, _, cp in cases],
                    implicit=dict(imp, max_iter=400, restart_projected=40), **kw)
    b.set_state(bad)
    b.set_fallback(q0)
    r = b.solve()
    st, qb = b.case_status(), b.state()
    b.close()
    assert r["n_restarted"] == len(cases) and np.all(st["restart_iter"] == 120)
    assert r["iterations"] == 400 and np.all(st["conv_iter"] == -1)
    for k in range(len(cases)):
        assert np.array_equal(qb[k], qc[k]), k


@pytest.mark.gpu
def test_gpu_batch_stalled_cases_retire_or_restart_once():
    """The stall test: with a 2-iteration window every case stalls within a
    few graph launches and is retired (MST_CASE_STALLED, no further cost);
    with fallback states each case first restarts from them, once, then
    stalls again."""
    from mstcfd import batch, capi
    from mstcfd import meshgen as mg
    cases = _batch_cases(0)
    q0 = [mg.freestream(mach, mesh.n_cells) for _, mesh, mach, _ in cases]
    b = batch.Batch([(mesh, cp) for _, mesh, _, cp in cases],
                    implicit=dict(stall_window=2, max_iter=4000),
                    flux=1, order=2, limiter=1, precision=1)
    b.set_state(q0)
    r = b.solve()
    st = b.case_status()
    assert r["n_stalled"] == len(cases) and r["n_converged"] == 0 and r["n_restarted"] == 0
    assert np.all(st["conv_iter"] == capi.CASE_STALLED) and r["iterations"] < 500
    assert np.all(st["restart_iter"] == -1)
    b.set_state(q0)
    b.set_fallback(q0)
    r = b.solve()
    st = b.case_status()
    assert r["n_restarted"] == len(cases) and r["n_stalled"] == len(cases)
    assert np.all(st["restart_iter"] > 0) and r["iterations"] < 1000
    with pytest.raises(capi.MstError):
        b.set_fallback(None)
        b.restart([0])
    b.close()


@pytest.mark.gpu
@pytest.mark.parametrize("fp32_until", [0.0, 1e-3], ids=["fp64_residual", "mixed_residual"])
def test_gpu_batch_fp32_sweeps_reach_tolerance(fp32_until):
    """FP32 sweeps (FP64 diagonal inversion and state update): every case
    reaches the same 1e-8 tolerance of the FP64 residual, and the converged
    fields agree with the FP64-sweep solve (the limiter freezes at a
    different iteration, hence an RMS rather than a round-off bound)."""
    from mstcfd import batch
    from mstcfd import meshgen as mg
    cases = _batch_cases(0)
    q0 = [mg.freestream(mach, mesh.n_cells) for _, mesh, mach, _ in cases]
    out = {}
    for sw in (0, 1):
        b = batch.Batch([(mesh, cp) for _, mesh, _, cp in cases],
                        implicit=dict(fp32_until=fp32_until, sweep_fp32=sw, max_iter=4000),
                        flux=1, order=2, limiter=1, precision=1)
        b.set_state(q0)
        r = b.solve()
        assert r["n_converged"] == len(cases), sw
        st = b.case_status()
        assert np.all(st["last_l2"] <= 1e-8 * st["first_l2"] * 1.0001)
        out[sw] = b.state()
        b.close()
    for a, c in zip(out[0], out[1]):
        rms = np.sqrt(np.mean((a - c) ** 2)) / np.sqrt(np.mean(a ** 2))
        assert rms < 1e-3


@pytest.mark.gpu
def test_gpu_batch_reference_l2_sets_the_tolerance():
    """With a caller-set reference L2 the tolerance, SER CFL and freezing
    measure against it: a reference equal to the first-iteration L2 gives
    the plain solve bit-for-bit; with a 10x larger one every case meets the
    correspondingly looser absolute target."""
    from mstcfd import batch
    from mstcfd import meshgen as mg
    cases = _batch_cases(0)
    q0 = [mg.freestream(mach, mesh.n_cells) for _, mesh, mach, _ in cases]
    kw = dict(flux=1, order=2, limiter=1, precision=1)
    imp = dict(max_iter=3000, graph_iters=10)
    b = batch.Batch([(mesh, cp) for _, mesh, _, cp in cases], implicit=imp, **kw)
    b.set_state(q0)
    b.solve()
    st = b.case_status()
    q_plain = b.state()
    b.set_state(q0)
    b.set_l2_ref(st["first_l2"])
    b.solve()
    st2 = b.case_status()
    assert np.array_equal(st2["conv_iter"], st["conv_iter"])
    for a, c in zip(b.state(), q_plain):
        assert np.array_equal(a, c)
    b.set_state(q0)
    b.set_l2_ref(10.0 * st["first_l2"])
    b.solve()
    st3 = b.case_status()
    assert np.all(st3["conv_iter"] >= 0)
    assert np.all(st3["last_l2"] <= 1e-8 * 10.0 * st["first_l2"] * 1.0001)
    b.close()
