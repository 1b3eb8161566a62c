"""Benchmark of the density-based residual path on GB300.

Workload (the 2D isentropic-vortex configuration): periodic [0,10]^2,
jittered Delaunay triangles from an n x n node lattice (n = 1000: 2,000,000
cells, 3,000,000 faces; node jitter U(-0.25h, 0.25h), seed 20261203),
vortex of strength 5 convected at Mach 0.5, AUSM+ flux, van Leer limiter,
two-stage Runge-Kutta at global CFL 0.5.  A step is one RK2 time step
(two residual evaluations and two state updates of every cell), i.e. two
cell-updates per cell.  Inputs (state + mesh, ~0.5 GB) exceed the 129 MB L2
between steps.

Arms:
  (default)          the CUDA path through the C ABI; value = FP32-flux /
                     float-pair-accumulate Mcell-updates/s (state and
                     residual sums as unevaluated FP32 pairs, no FP64
                     instruction) with the state resident
                     in HBM, timed with CUDA events on the context's stream;
                     "fp64" = the same in FP64 (with its FP64-pipe
                     roofline); "e2e" = FP32 through the public API with
                     host buffers: each step a job of mst_step_host_jobs,
                     its state copied host->device and back (page-locked
                     buffers), the copies overlapped with the neighbouring
                     jobs' computation.
  --impl reference   the CPU restatement of the same path (the oracle,
                     OpenMP over all host cores) on the same workload.

The line also carries "batch": the batched steady-wedge family (the
compression-ramp cases of mstcfd.meshgen.wedge_family: seeded Mach U[1.5,3],
ramp angle U[5,15] deg redrawn while the inviscid post-shock Mach is below
1.2, Re U[1e3,1e4], laminar, Roe + minmod) solved from free stream (cold
start) to L2 1e-8 by the batched LU-SGS path in FP64 and with the
production options -- wall time of the whole batch, iterations, cases
converged -- and from the learned initial field with the same options
(batch.warm); --batch-cases and --batch-cells set its size (0 cases:
skipped); "tgv3d" the 3D Taylor-Green vortex; "simple" the pressure-based
SIMPLE solver.

One JSON line on rank 0.  Under torchrun each rank runs an independent
replica on its own GPU (single-mesh runs do not shard: replicas only).
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "mst-cfd_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "Mcell-updates/s FP32 vs FP64"
UNIT = "Mcell-updates/s"


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class _Group:
    """Barrier and max-reduce across ranks (gloo; no data-path collective)."""

    def __init__(self, ws):
        self.ws = ws
        self.dist = None
        if ws > 1:
            import torch.distributed as dist
            dist.init_process_group("gloo")
            self.dist = dist

    def barrier(self):
        if self.dist:
            self.dist.barrier()

    def max(self, x):
        if not self.dist:
            return x
        import torch
        t = torch.tensor([float(x)], dtype=torch.float64)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def sum(self, x):
        if not self.dist:
            return x
        import torch
        t = torch.tensor([float(x)], dtype=torch.float64)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.SUM)
        return float(t.item())


class _Clocks:
    """nvidia-smi clock / throttle sampling during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows = []
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 8:
                continue
            try:
                rows.append((float(f[0]), float(f[1]), f[4:8]))
            except ValueError:
                continue
        os.unlink(self.path)
        if not rows:
            return None
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for _, _, r in rows for i, v in enumerate(r)
                          if v.lower().startswith("active")})
        return {"sm_mhz": statistics.median(r[0] for r in rows),
                "sm_max_mhz": max(r[1] for r in rows), "reasons": reasons,
                "samples": len(rows)}


def _workload(n):
    from mstcfd import meshgen as mg
    m = mg.periodic_delaunay(n, 10.0, jitter=0.25, seed=20261203)
    return m


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def _tensor_peak():
    """Burst dense BF16 TFLOP/s (the GEMMs are timed alone)."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["bf16_tflops"]), "measured"
    except Exception:
        return 1900.0, "fallback"


def _gemm_at_scale(net, feats):
    """One forward + backward of the network over the union of the batch's
    graphs with every tensor-core GEMM launch timed by CUDA events: achieved
    TFLOP/s (2MNK) and GB/s (operands + results) against the measured
    peaks."""
    from mstcfd import warmstart as ws
    fu, pu, nu, _ = ws.union([(f, ptr, nbr, None) for f, ptr, nbr, _ in feats])
    net.set_graph(fu, pu, nu)
    net.set_targets(np.zeros((len(fu), 4), np.float32))
    net.forward()
    net.backward()  # warm-up
    net.profile(True)
    t0 = time.perf_counter()
    net.forward()
    net.backward()
    step_s = time.perf_counter() - t0
    g = net.profile_read()
    net.profile(False)
    tf_peak, tf_src = _tensor_peak()
    hbm, hbm_src = _peaks()
    tflops = g["flops"] / (g["ms"] * 1e-3) / 1e12
    gbs = g["bytes"] / (g["ms"] * 1e-3) / 1e9
    ridge = tf_peak * 1e12 / (hbm * 1e9)
    return {"cells": int(len(fu)), "train_step_s": round(step_s, 4),
            "gemm_launches": g["launches"], "gemm_ms": round(g["ms"], 3),
            "gemm_share_of_step": round(g["ms"] * 1e-3 / step_s, 3),
            "tflops": round(tflops, 2), "tensor_frac": round(tflops / tf_peak, 4),
            "tensor_peak": tf_peak, "tensor_peak_source": tf_src,
            "gbs": round(gbs, 1), "hbm_frac": round(gbs / hbm, 4), "hbm_peak_source": hbm_src,
            "flops_per_byte": round(g["flops"] / g["bytes"], 1),
            "ridge_flops_per_byte": round(ridge, 1),
            "bound": "hbm" if g["flops"] / g["bytes"] < ridge else "tensor"}


def _profile_traffic(kernel, n_cells):
    """DRAM bytes per launch of ``kernel`` from the committed ncu summary
    (per cell, scaled to this mesh), or None."""
    path = os.path.join(ROOT, "profiles", "flux_update_gradient_vortex2M_ncu.txt")
    if not os.path.exists(path):
        return None
    for line in open(path):
        if line.startswith("dram_bytes_per_cell[" + kernel + "]"):
            try:
                return float(line.split("=")[1].split()[0]) * n_cells
            except (IndexError, ValueError):
                return None
    return None


_FP64_PROFILE = os.path.join(ROOT, "profiles", "fp64_pipe_vortex_tgv_ncu.txt")


def _fp64_counts(kernel):
    """FP64-pipe thread instructions (DADD + DMUL + DFMA) and flops (DFMA
    counted twice) per cell of one launch of ``kernel``, from the committed
    ncu instruction counts, or None."""
    if not os.path.exists(_FP64_PROFILE):
        return None
    out = {}
    for line in open(_FP64_PROFILE):
        for key in ("fp64_inst_per_cell", "fp64_flops_per_cell"):
            if line.startswith(f"{key}[{kernel}]"):
                try:
                    out[key] = float(line.split("=")[1].split()[0])
                except (IndexError, ValueError):
                    pass
    return out if len(out) == 2 else None


_FP64_RATE = None


def _fp64_rate():
    """Measured FP64 FMA rate of this GPU (thread instructions / s)."""
    global _FP64_RATE
    if _FP64_RATE is None:
        import ctypes as C
        from mstcfd import capi
        r = C.c_double()
        capi.check(capi.load().mst_probe_fp64_rate(C.byref(r)))
        _FP64_RATE = r.value
    return _FP64_RATE


def _fp64_roofline(kernel, n_cells, avg_ms, prof):
    """The FP64 arm's dominant kernel against the FP64 pipe: its FP64
    instructions per launch (ncu counts per cell x cells) over its live
    average launch time, against the DFMA rate measured by a probe kernel."""
    cnt = _fp64_counts(kernel)
    rate = _fp64_rate()
    if cnt is None:
        return {"bound": "fp64", "kernel": kernel, "achieved": None,
                "note": "no committed FP64 instruction counts for this kernel"}
    inst = cnt["fp64_inst_per_cell"] * n_cells
    flops = cnt["fp64_flops_per_cell"] * n_cells
    ach = inst / (avg_ms * 1e-3)
    return {"bound": "fp64", "kernel": kernel, "achieved": round(ach / 1e12, 4),
            "peak": round(rate / 1e12, 4), "unit": "T FP64-inst/s", "frac": round(ach / rate, 4),
            "peak_source": "measured (DFMA probe kernel, mst_probe_fp64_rate)",
            "gflops": round(flops / (avg_ms * 1e-3) / 1e9, 1),
            "peak_gflops": round(2 * rate / 1e9, 1),
            "fp64_inst_per_cell_launch": cnt["fp64_inst_per_cell"],
            "fp64_flops_per_cell_launch": cnt["fp64_flops_per_cell"],
            "counts_source": os.path.relpath(_FP64_PROFILE, ROOT),
            "avg_launch_ms": round(avg_ms, 4),
            "kernel_share": {k: round(v[1] / sum(x[1] for x in prof.values()), 4)
                             for k, v in prof.items()}}


def run_gpu(args, ws, rank, local, grp):
    from mstcfd import Mesh, PinnedArray, Solver, capi, roofline
    from mstcfd import meshgen as mg
    capi.check(capi.load().mst_set_device(local))
    m = _workload(args.n)
    mesh = Mesh.from_arrays(m["node_xy"], m["face_nodes"], m["face_cells"], m["zones"],
                            m["n_cells"], c1_shift=m["c1_shift"])
    nC = mesh.n_cells
    q0 = mg.isentropic_vortex(m["cell_centroid"])
    kw = dict(flux=0, order=2, limiter=2, reference_quirks=0, time_scheme=1,
              dt_mode=1, cfl=0.5)
    results = {}
    prof = {}
    for prec, label in ((2, "fp32"), (1, "fp64")):
        steps = args.steps if prec == 2 else max(3, args.steps // 4)
        s = Solver(mesh, precision=prec, **kw)
        s.set_state(q0)
        s.step(args.warmup)
        clocks = _Clocks(local) if prec == 2 else None
        grp.barrier()
        if clocks:
            clocks.start()
        s.profile(True)
        s.step(steps)
        ms, launches = s.last_timing()
        s.profile(False)
        if clocks:
            results["clocks"] = clocks.stop()
        grp.barrier()
        ms_max = grp.max(ms)
        cells_all = grp.sum(2.0 * nC * steps)
        results[label] = dict(value=cells_all / (ms_max * 1e-3) / 1e6,
                              ms_per_step=ms_max / steps, steps=steps,
                              launches=launches)
        prof[label] = s.profile_stats()
        if prec == 2:
            # end to end through the public API with host buffers: every
            # step is a job whose state comes from page-locked host memory
            # and goes back to it (mst_step_host_jobs: the copies of the
            # neighbouring jobs overlap this job's computation)
            hin = [PinnedArray((nC, 4)) for _ in range(2)]
            hout = [PinnedArray((nC, 4)) for _ in range(2)]
            for h in hin:
                h.array[:] = s.state()
            ins = [hin[j % 2].ptr.value for j in range(steps)]
            outs = [hout[j % 2].ptr.value for j in range(steps)]
            s.step_host_jobs(ins[:2], outs[:2], nsteps=1)  # warm-up (pipeline set-up)
            grp.barrier()
            t0 = time.perf_counter()
            s.step_host_jobs(ins, outs, nsteps=1)
            t1 = time.perf_counter()
            grp.barrier()
            e2e_s = grp.max(t1 - t0)
            results["e2e"] = dict(value=cells_all / e2e_s / 1e6, unit=UNIT,
                                  h2d_bytes_per_step=int(hin[0].nbytes),
                                  d2h_bytes_per_step=int(hout[0].nbytes),
                                  api="mst_step_host_jobs (one job = one RK2 step of a "
                                      "host-held state; copies overlapped)")
            if not all(np.all(np.isfinite(h.array)) for h in hout):
                raise RuntimeError("non-finite state after the e2e steps")
            for h in hin + hout:
                h.free()
        s.close()
    # roofline of the dominant kernel (largest share of the FP32 step)
    st = prof["fp32"]
    top = max(st, key=lambda k: st[k][1])
    n_launch, tot_ms = st[top]
    avg_ms = tot_ms / n_launch
    info = mesh.info
    if top.startswith("k_flux_update"):
        # launches alternate stage 0 / stage 1
        b = 0.5 * (roofline.kernel_bytes(info, 2, 2, top, stage=0) +
                   roofline.kernel_bytes(info, 2, 2, top, stage=1))
    else:
        b = roofline.kernel_bytes(info, 2, 2, top)
    peak, peak_kind = _peaks()
    achieved = b / (avg_ms * 1e-3) / 1e9
    traffic = _profile_traffic(top, nC)
    share = {k: round(v[1] / sum(x[1] for x in st.values()), 4) for k, v in st.items()}
    # the FP64 arm against the FP64 pipe (its bound) and, beside it, HBM
    s64 = prof["fp64"]
    top64 = max(s64, key=lambda k: s64[k][1])
    avg64 = s64[top64][1] / s64[top64][0]
    results["fp64"]["roofline"] = _fp64_roofline(top64, nC, avg64, s64)
    if top64.startswith("k_flux_update"):
        b64 = 0.5 * (roofline.kernel_bytes(info, 1, 2, top64, stage=0) +
                     roofline.kernel_bytes(info, 1, 2, top64, stage=1))
        results["fp64"]["roofline_hbm"] = {
            "bound": "hbm", "kernel": top64, "achieved": round(b64 / (avg64 * 1e-3) / 1e9, 1),
            "peak": _peaks()[0], "unit": "GB/s",
            "frac": round(b64 / (avg64 * 1e-3) / 1e9 / _peaks()[0], 4)}
    return results, dict(bound="hbm", achieved=round(achieved, 1), peak=peak,
                         unit="GB/s", frac=round(achieved / peak, 4),
                         traffic=traffic, kernel=top, peak_source=peak_kind,
                         algorithmic_bytes_per_launch=int(b),
                         avg_launch_ms=round(avg_ms, 5), kernel_share=share), nC


def _ramp_mesh(p):
    from mstcfd import meshgen as mg
    return mg.wedge(p["cells"], p["angle"], seed=p["seed"])


def _ramp_meshes(fam):
    """The ramp meshes of a family, generated on the host's cores (fresh
    interpreters: nothing of this process's CUDA state is inherited)."""
    import multiprocessing as mp
    from concurrent.futures import ProcessPoolExecutor
    workers = min(16, os.cpu_count() or 1, len(fam))
    if workers <= 1:
        return [_ramp_mesh(p) for p in fam]
    with ProcessPoolExecutor(workers, mp_context=mp.get_context("spawn")) as ex:
        return list(ex.map(_ramp_mesh, fam, chunksize=4))


def _wedge_cases(n_cases, lo, hi):
    """Seeded compression-ramp family: (mesh dict, Mach, angle, Re)."""
    from mstcfd import meshgen as mg
    fam = mg.wedge_family(n_cases, cells=(lo, hi))
    return [(m, p["mach"], p["angle"], p["reynolds"]) for m, p in zip(_ramp_meshes(fam), fam)]


# temperature floor of the batched LU-SGS solves, p >= P_FLOOR rho (1.4% of
# the free stream's p / rho): a near-vacuum cell at the slip / no-slip
# corner of a ramp otherwise rejects every update and freezes its case
P_FLOOR = 0.01


def _production(args):
    """Implicit parameters of the batch's production runs (warm start and
    the matching cold start)."""
    return dict(max_iter=args.batch_iters, fp32_until=args.fp32_until, sweep_fp32=1,
                p_floor=P_FLOOR, fp32_window=args.fp32_window, stall_window=STALL_WINDOW)


def _production_label(args):
    return (f"FP32 residual until each case's L2 is {args.fp32_until:g} of its first (or "
            f"stagnates for {args.fp32_window} iterations), then FP64, case by case; FP32 "
            f"sweeps, FP64 diagonal inversion and update")


def _case_info(mesh, case):
    """Cells and flow parameters of one ramp case (mesh, (m, mach, angle, re))."""
    from mstcfd import meshgen as mg
    _, mach, angle, re = case
    return {"cells": int(mesh.n_cells), "mach": round(float(mach), 4),
            "angle": round(float(angle), 4), "reynolds": round(float(re), 1),
            "post_shock_mach": round(float(mg.post_shock_mach(mach, angle) or 0.0), 3)}


def _batch_solve(cases, q0, imp, grp, l2_ref=None, fallback=None):
    """One batched LU-SGS solve (FP64 production path: Roe + minmod,
    laminar): wall time (max over ranks), result, per-case status, states.
    fallback: states a stalled case restarts from within the solve."""
    from mstcfd import batch
    b = batch.Batch(cases, implicit=imp, flux=1, order=2, limiter=1, precision=1, viscous=1)
    b.set_state(q0)
    if l2_ref is not None:
        b.set_l2_ref(l2_ref)
    if fallback is not None:
        b.set_fallback(fallback)
    grp.barrier()
    t0 = time.perf_counter()
    r = b.solve()
    wall = time.perf_counter() - t0
    grp.barrier()
    st = b.case_status()
    info = b.info()
    q = b.state()
    b.close()
    return grp.max(wall), r, st, info, q


# a case whose L2 has not halved for this many iterations of its FP64 phase
# is retired as stalled (restarted from the free stream where a warm start
# set it as the fallback)
STALL_WINDOW = 3000


def _fp64_opts(args):
    return dict(max_iter=args.batch_iters, p_floor=P_FLOOR, stall_window=STALL_WINDOW)


def run_batch(args, ws, rank, grp):
    """Cold-start batched LU-SGS solve of the wedge family to L2 1e-8.  With
    N ranks the cases are split by greedy size balancing, each rank solves
    its share on its own GPU (no exchange), and the wall time is the
    maximum over ranks."""
    from mstcfd import Mesh, batch
    from mstcfd import meshgen as mg
    gamma, cv = 1.4, 1.0 / (1.4 * 0.4)
    fam = _wedge_cases(args.batch_cases, args.batch_cells[0], args.batch_cells[1])
    mine = batch.partition_cases([m["n_cells"] for m, _, _, _ in fam], ws)[rank]
    fam = [fam[i] for i in mine]
    cases, q0 = [], []
    for m, mach, angle, re in fam:
        mesh = Mesh.from_arrays(m["node_xy"], m["face_nodes"], m["face_cells"], m["zones"],
                                m["n_cells"])
        mu = mach / re
        cases.append((mesh, batch.case_params(mg.freestream(mach), mu=mu, lambda_=-2 / 3 * mu,
                                              kappa=mu * gamma * cv / 0.72, cv=cv)))
        q0.append(mg.freestream(mach, mesh.n_cells))
    wall, r, st, info, q_cold = _batch_solve(cases, q0, _fp64_opts(args), grp)
    cells = int(sum(m.n_cells for m, _ in cases))
    conv = st["conv_iter"]
    n_conv = int(grp.sum((conv >= 0).sum()))
    cells_all = int(grp.sum(cells))
    out = {"metric": "batch time to L2 res 1e-8 (cold start, FP64)", "unit": "s",
           "value": round(wall, 3), "device_s": round(r["ms"] * 1e-3, 3),
           "cases": args.batch_cases, "cells": cells_all, "converged": n_conv,
           "diverged": int(grp.sum(r["n_diverged"])),
           "stalled": int(grp.sum(r["n_stalled"])),
           "partition": "greedy size balancing over ranks, no exchange",
           "iterations": r["iterations"], "max_iter": args.batch_iters,
           "median_case_iterations": int(np.median(conv[conv >= 0])) if (conv >= 0).any() else None,
           "Mcell_iterations_per_s": round(cells * r["iterations"] / (r["ms"] * 1e-3) / 1e6, 1),
           # the work actually done: each case's cells times the iterations
           # it ran (a converged case costs nothing afterwards)
           "case_Mcell_iterations_per_s": round(
               sum(m.n_cells * (int(c) + 1 if c >= 0 else r["iterations"])
                   for (m, _), c in zip(cases, conv)) / (r["ms"] * 1e-3) / 1e6, 1),
           "colors": info["n_colors"], "sweep_threads": info["sweep_threads"],
           "graph_iters": info["graph_iters"],
           # the cases left at the cap (at most 16): cells, flow parameters,
           # L2 / first L2
           "not_converged": [dict(_case_info(cases[i][0], fam[i]), case=int(mine[i]),
                                  l2_ratio=float(st["last_l2"][i] / st["first_l2"][i]))
                             for i in range(len(cases)) if conv[i] < 0][:16],
           "workload": (f"{len(cases)} compression ramps (no-slip flat plate and ramp), "
                        f"{args.batch_cells[0]}-"
                        f"{args.batch_cells[1]} triangles each, Mach U[1.5,3], angle U[5,15] deg "
                        f"(redrawn while the inviscid post-shock Mach is below 1.2), "
                        f"Re U[1e3,1e4] laminar, Roe + minmod, LU-SGS, temperature floor p >= "
                        f"{P_FLOOR} rho, cap "
                        f"{args.batch_iters} iterations, a case whose L2 has not halved in "
                        f"{STALL_WINDOW} iterations retired as stalled"),
           "warm": None}
    first_cold = st["first_l2"]
    # the same cold start with the production options
    wall_m, rm, stm, _, _ = _batch_solve(cases, q0, _production(args), grp)
    cm = stm["conv_iter"]
    out["cold_mixed"] = {"value": round(wall_m, 3), "unit": "s",
                         "converged": int(grp.sum((cm >= 0).sum())),
                         "stalled": int(grp.sum(rm["n_stalled"])),
                         "iterations": rm["iterations"],
                         "median_case_iterations": int(np.median(cm[cm >= 0]))
                         if (cm >= 0).any() else None,
                         "not_converged": [dict(_case_info(cases[i][0], fam[i]),
                                                case=int(mine[i]), l2_ratio=float(stm["last_l2"][i]
                                                               / stm["first_l2"][i]))
                                           for i in range(len(cases)) if cm[i] < 0][:16],
                         "precision": _production_label(args)}
    if args.warm_train > 0:
        out["warm"] = run_warm(args, fam, cases, q0, q_cold, conv, first_cold, cm, wall,
                               wall_m, grp)
    return out


def run_warm(args, fam, cases, q_free, q_cold, conv_cold, first_cold, conv_cold_m, wall_cold,
             wall_cold_m, grp):
    """Learned warm start of the same batch: the network is trained on the
    GPU (tensor-core forward/backward) on ramps of a disjoint seed range
    that the batched solver converged from free stream, then predicts the
    initial fields; the batch is solved again from them, with the same
    options as each cold start and held to the cold start's absolute
    residual target per case.  A warm-started case that does not reach it
    within the cap is solved again from free stream (the fallback), and
    that time is added.  Final fields are compared with the cold start's."""
    from mstcfd import Mesh, warmstart as ws
    from mstcfd import meshgen as mg
    from mstcfd.mpnn import Network
    t0 = time.perf_counter()
    train = []
    # ramps of the batch's own size range (a network trained on coarser
    # ramps of 4k-12k cells gained nothing on these), seeds disjoint
    tfam = mg.wedge_family(args.warm_train, cells=tuple(args.batch_cells), seed=777)
    for p, m in zip(tfam, _ramp_meshes(tfam)):
        cp = ws.case_params_of(p)
        mesh = Mesh.from_arrays(m["node_xy"], m["face_nodes"], m["face_cells"], m["zones"],
                                m["n_cells"])
        train.append((p, m, mesh, cp))
    # training data: the batched solver's own converged solutions (cold
    # start, production options, the same 1e-8 tolerance)
    _, _, tst, _, tq = _batch_solve([(mesh, cp) for _, _, mesh, cp in train],
                                    [mg.freestream(p["mach"], mesh.n_cells)
                                     for p, _, mesh, _ in train], _production(args), grp)
    tconv = tst["conv_iter"]
    samples = []
    for k, (p, m, mesh, _) in enumerate(train):
        if tconv[k] >= 0:
            ptr, nbr = ws.neighbours(m)
            samples.append((ws.features(m, mesh.arrays(), p), ptr, nbr,
                            ws.targets(tq[k], p["mach"])))
    data_s = time.perf_counter() - t0
    if not samples:
        return {"value": None, "note": f"no training case converged within "
                                        f"{args.batch_iters} iterations"}
    net = Network(seed=11)
    t1 = time.perf_counter()
    hist = ws.train(net, samples, steps=args.warm_steps, lr=2e-3, per_step=4)
    train_s = time.perf_counter() - t1
    feats = []
    for (m, mach, angle, re), (mesh, _) in zip(fam, cases):
        p = dict(mach=mach, angle=angle, reynolds=re)
        ptr, nbr = ws.neighbours(m)
        feats.append((ws.features(m, mesh.arrays(), p), ptr, nbr, mach))
    grp.barrier()
    t2 = time.perf_counter()
    q_warm = [ws.state(ws.predict(net, f, ptr, nbr), mach) for f, ptr, nbr, mach in feats]
    infer_s = time.perf_counter() - t2
    gemm = _gemm_at_scale(net, feats)
    net.close()

    # a warm case that stalls restarts from the free stream inside the
    # solve (its fallback); its iterations count from the warm start.  (An
    # iteration budget as the trigger -- restart_after at the 90th
    # percentile of the training solves' iterations, 10,346 -- restarted
    # cases that were slow but converging and cost more than it saved.)

    def warm_run(opts, conv_c, wall_c, label):
        # ... or whose L2, at its rate over two 1,000-iteration windows in a
        # row, would not reach the tolerance within the cap
        wall, r, st, _, qw = _batch_solve(cases, q_warm, dict(opts, restart_projected=1000),
                                          grp, l2_ref=first_cold, fallback=q_free)
        conv = st["conv_iter"]
        # cases still not at the tolerance are solved again from free
        # stream, to the same tolerance, and that time is added
        miss = [k for k in range(len(cases)) if conv[k] < 0]
        fb_s, fb_conv = 0.0, 0
        if miss:
            fb_s, _, fst, _, fq = _batch_solve([cases[k] for k in miss],
                                               [q_free[k] for k in miss], opts, grp)
            fb_conv = int((fst["conv_iter"] >= 0).sum())
            for i, k in enumerate(miss):
                qw[k] = fq[i]
        total = infer_s + wall + fb_s
        both = [k for k in range(len(cases)) if conv[k] >= 0 and conv_c[k] >= 0]
        it_w = [int(conv[k]) for k in both]
        it_c = [int(conv_c[k]) for k in both]
        n_ok = int((conv >= 0).sum()) + fb_conv
        res = {"value": round(total, 3), "unit": "s", "precision": label,
               "solve_s": round(wall, 3), "inference_s": round(infer_s, 3),
               "converged": int(grp.sum(n_ok)), "converged_warm": int(grp.sum((conv >= 0).sum())),
               "restarted_in_solve": int(grp.sum(r["n_restarted"])),
               "restart_iterations": [int(x) for x in st["restart_iter"] if x >= 0],
               "fallback_cases": len(miss), "fallback_s": round(fb_s, 3),
               "iterations": r["iterations"],
               "iteration_ratio_cold_over_warm": round(float(np.sum(it_c)) / max(np.sum(it_w), 1), 3)
               if it_c else None,
               "case_iterations": {"cold": [int(x) for x in conv_c], "warm": [int(x) for x in conv]},
               "speedup_vs_cold_same_options": round(wall_c / total, 3)}
        ok = [k for k in range(len(cases)) if conv_c[k] >= 0]
        if ok:
            res["max_rms_rel_field_diff_vs_cold"] = max(
                float(np.sqrt(np.mean((qw[k] - q_cold[k]) ** 2)) / np.sqrt(np.mean(q_cold[k] ** 2)))
                for k in ok)
            res["max_rel_field_diff_vs_cold"] = max(
                float(np.abs(qw[k] - q_cold[k]).max() / np.abs(q_cold[k]).max()) for k in ok)
        return res

    warm64 = warm_run(_fp64_opts(args), conv_cold, wall_cold,
                      "FP64 residual and sweeps (the plain cold start's options)")
    warm_m = warm_run(_production(args), conv_cold_m, wall_cold_m, _production_label(args))
    return {"tolerance": "L2 <= 1e-8 x the cold start's first-iteration L2 of each case "
                         "(the same absolute residual as the cold start)",
            "fp64": warm64, "production": warm_m,
            "speedup_same_options": {"fp64": warm64["speedup_vs_cold_same_options"],
                                     "production": warm_m["speedup_vs_cold_same_options"]},
            "warm_production_vs_plain_fp64_cold": round(wall_cold / warm_m["value"], 3),
            "train": {"cases": args.warm_train, "converged": len(samples),
                      "cells": f"{args.batch_cells[0]}-{args.batch_cells[1]}",
                      "seeds": "disjoint from the batch", "steps": args.warm_steps,
                      "loss_first": round(float(hist[0]), 5),
                      "loss_last": round(float(hist[-20:].mean()), 5),
                      "loss_curve": [round(float(hist[i:i + 50].mean()), 5)
                                     for i in range(0, len(hist), max(1, len(hist) // 8))],
                      "data_s": round(data_s, 2), "train_s": round(train_s, 2)},
            "network_gemm": gemm}


def run_network_only(args):
    """Network GEMMs over the batch's cases (features of the ramp family)."""
    from mstcfd import Mesh, warmstart as ws
    from mstcfd.mpnn import Network
    fam = _wedge_cases(args.batch_cases, args.batch_cells[0], args.batch_cells[1])
    feats = []
    for m, mach, angle, re in fam:
        mesh = Mesh.from_arrays(m["node_xy"], m["face_nodes"], m["face_cells"], m["zones"],
                                m["n_cells"])
        ptr, nbr = ws.neighbours(m)
        feats.append((ws.features(m, mesh.arrays(), dict(mach=mach, angle=angle, reynolds=re)),
                      ptr, nbr, mach))
    net = Network(seed=11)
    out = _gemm_at_scale(net, feats)
    net.close()
    return out


def run_cpu_sample(m, steps, budget_s=30.0):
    """The oracle port (OpenMP over all host cores) on the workload."""
    from mstcfd import meshgen as mg
    from oracle import pyoracle as po
    om = po.mesh_from_arrays(m["node_xy"], m["face_nodes"], m["face_cells"], m["zones"],
                             m["n_cells"], c1_shift=m["c1_shift"])
    q = mg.isentropic_vortex(m["cell_centroid"])
    prm = po.params_ext(0, 2, limiter=2, quirks=0, rk2=1, dt_mode=1, cfl=0.5)
    q, _ = po.step_ext(om, prm, q, 1)  # warm
    done, t_total = 0, 0.0
    while done < steps:
        t0 = time.perf_counter()
        q, _ = po.step_ext(om, prm, q, 1)
        t_total += time.perf_counter() - t0
        done += 1
        if t_total > budget_s:
            break
    cores = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    return 2.0 * m["n_cells"] * done / t_total / 1e6, cores, done, t_total


def run_batch_scale(args, grp):
    """Throughput of the batched LU-SGS at a larger batch (a fixed number
    of iterations, FP64 residual and sweeps, no convergence target): the
    Mcell-iterations/s the cold-start path sustains at config-4 scale."""
    from mstcfd import Mesh, batch
    from mstcfd import meshgen as mg
    gamma, cv = 1.4, 1.0 / (1.4 * 0.4)
    t0 = time.perf_counter()
    fam = _wedge_cases(args.scale_cases, args.scale_cells[0], args.scale_cells[1])
    cases, q0 = [], []
    for m, mach, angle, re in fam:
        mesh = Mesh.from_arrays(m["node_xy"], m["face_nodes"], m["face_cells"], m["zones"],
                                m["n_cells"])
        mu = mach / re
        cases.append((mesh, batch.case_params(mg.freestream(mach), mu=mu, lambda_=-2 / 3 * mu,
                                              kappa=mu * gamma * cv / 0.72, cv=cv)))
        q0.append(mg.freestream(mach, mesh.n_cells))
    setup_s = time.perf_counter() - t0
    cells = int(sum(m.n_cells for m, _ in cases))
    out = {"cases": args.scale_cases, "cells": cells, "cell_range": list(args.scale_cells),
           "mesh_setup_s": round(setup_s, 1)}
    # the cold-start path (FP64 residual and sweeps) and the production
    # options (FP32 residual -- the FP32 phase lasts the whole short run --
    # and FP32 sweeps)
    for label, imp in (("fp64", dict(p_floor=P_FLOOR)),
                       ("production", dict(fp32_until=args.fp32_until, sweep_fp32=1,
                                           fp32_window=args.fp32_window,
                                           p_floor=P_FLOOR))):
        b = batch.Batch(cases, implicit=dict(imp, max_iter=args.scale_iters, tol=1e-30),
                        flux=1, order=2, limiter=1, precision=1, viscous=1)
        b.set_state(q0)
        grp.barrier()
        r = b.solve()
        info = b.info()
        b.close()
        out[label] = {"iterations": r["iterations"], "device_s": round(r["ms"] * 1e-3, 3),
                      "Mcell_iterations_per_s": round(cells * r["iterations"]
                                                      / (r["ms"] * 1e-3) / 1e6, 1),
                      "colors": info["n_colors"], "sweep_threads": info["sweep_threads"]}
    return out


def run_tgv3d(args, grp):
    """3D Taylor-Green vortex (Ma 0.1, Re 1600, laminar) on the periodic
    jittered Kuhn tetrahedral mesh of (tgv_n)^3 x 6 cells: FP32 and FP64
    Mcell-updates/s of RK2 steps (Roe + van Albada + viscous term, CFL 0.5),
    the dominant kernel against the HBM roofline, and the CPU restatement
    timed on a bounded sample of the same family."""
    from mstcfd import meshgen as mg
    from mstcfd import roofline as rl
    from mstcfd.mesh3d import Mesh3D
    from mstcfd.solver3d import Solver3D
    n = args.tgv_n
    t0 = time.perf_counter()
    m = mg.tet_grid(n, jitter=0.15, seed=20261205)
    q0 = mg.taylor_green(m["cell_centroid"], mach=0.1)
    mesh = Mesh3D.from_dict(m)
    setup_s = time.perf_counter() - t0
    nC = int(m["n_cells"])
    mu = 0.1 / 1600.0  # rho V0 L / mu = 1600 with V0 = Ma 0.1 x a (= 1), L = 1
    cv = 1.0 / (1.4 * 0.4)
    kw = dict(order=2, limiter=3, viscous=1, mu=mu, lambda_=-2.0 / 3.0 * mu,
              kappa=mu * 1.4 * cv / 0.71, cv=cv, cfl=0.5)
    hbm, src = _peaks()
    out = {"workload": f"3D Taylor-Green vortex, Ma 0.1, Re 1600, periodic [0,2pi)^3, "
                       f"{n}^3 hexahedra x 6 jittered tetrahedra ({nC} cells), Roe + van "
                       f"Albada + laminar viscous term, RK2, CFL 0.5",
           "cells": nC, "faces": len(m["faces"]), "mesh_setup_s": round(setup_s, 1),
           "step": "one RK2 time step = 2 cell-updates per cell",
           "l2": "inputs larger than L2 (state + mesh ~10 GB)"}
    for prec, label in ((2, "fp32"), (1, "fp64")):
        s = Solver3D(mesh, precision=prec, **kw)
        info = s.info
        s.set_state(q0)
        ke0 = s.kinetic_energy()[0]
        s.step(max(3, args.warmup))
        steps = args.tgv_steps if prec == 2 else max(2, args.tgv_steps // 5)
        grp.barrier()
        s.step(steps)
        ms, launches = s.last_timing()
        ms = grp.max(ms)
        s.profile(True)
        s.step(steps)
        prof = s.profile_stats()
        s.profile(False)
        ke1 = s.kinetic_energy()[0]
        t = s.step(0)
        res = {"value": round(2 * nC * steps * grp.ws / (ms * 1e-3) / 1e6, 2),
               "unit": UNIT, "ms_per_step": round(ms / steps, 4), "steps": steps,
               "gpu_launches": launches, "device_gb": round(info["device_bytes"] / 1e9, 2),
               "kinetic_energy": {"t0": ke0, "t": t, "ratio": ke1 / ke0}}
        if "k3_flux_update" in prof:
            nl, tot_ms = prof["k3_flux_update"]
            by = 0.5 * sum(rl.kernel_bytes3d(nC, info["n_faces"], info["n_cell_faces"],
                                             info["n_tiles"], info["n_borrowed"], prec, 2, 1,
                                             "k3_flux_update", stage=st) for st in (0, 1))
            avg = tot_ms / nl
            if prec == 1:
                res["roofline"] = _fp64_roofline("k3_flux_update<f64>", nC, avg, prof)
            else:
                res["roofline"] = {
                    "bound": "hbm", "kernel": "k3_flux_update",
                    "achieved": round(by / (avg * 1e-3) / 1e9, 1), "peak": hbm,
                    "unit": "GB/s", "frac": round(by / (avg * 1e-3) / 1e9 / hbm, 4),
                    "peak_source": src, "algorithmic_bytes_per_launch": int(by),
                    "avg_launch_ms": round(avg, 4),
                    "kernel_share": {k: round(v[1] / sum(x[1] for x in prof.values()), 4)
                                     for k, v in prof.items()}}
            res["algorithmic_bytes_per_cell_update"] = round(
                rl.step_bytes3d(nC, info["n_faces"], info["n_cell_faces"], info["n_tiles"],
                                info["n_borrowed"], prec, 2, 1) / (2 * nC), 1)
        out[label] = res
        s.close()
    mesh.close()
    if args.no_cpu or grp.ws > 1:
        return out
    # CPU restatement (single thread) on a bounded sample of the same family
    from oracle import build as ob
    from oracle import pyoracle as po
    ob.build_oracle()
    ns = min(n, 48)
    ms_ = mg.tet_grid(ns, jitter=0.15, seed=20261205)
    om = po.Mesh3(ms_["node_xyz"], ms_["faces"], ms_["face_cells"], ms_["zones"],
                  ms_["n_cells"], ms_["c1_shift"])
    qs = mg.taylor_green(ms_["cell_centroid"], mach=0.1)
    p = po.params3(order=2, limiter=3, viscous=1, mu=mu, lam=-2.0 / 3.0 * mu,
                   kappa=mu * 1.4 * cv / 0.71, cv=cv)
    t1 = time.perf_counter()
    po.rk2_3(om, p, qs, 1, 0.5)
    secs = time.perf_counter() - t1
    out["cpu_baseline"] = {"value": round(2 * ms_["n_cells"] / secs / 1e6, 3), "unit": UNIT,
                           "cores": 1, "kind": "port",
                           "sample": f"1 RK2 step of the {ns}^3 x 6 = {ms_['n_cells']}-cell "
                                     f"mesh of the same family ({secs:.1f} s, FP64)"}
    return out


def run_simple(args, grp):
    """Pressure-based SIMPLE time steps (the reference's default solver:
    PSolver with SolverSIMPLE, 5 SIMPLE iterations per step, DT = 1/4000)
    on triangle channels with inlet, outlet and wall zones from the
    reference's initial field: time steps per second of mst_simple_step
    (one kernel launch per call, wall clock around the call), and the
    oracle's single-thread CPU time on the same meshes."""
    import tempfile
    from mstcfd import Mesh
    from mstcfd import meshgen as mg
    from mstcfd.psolver import SimpleSolver, reference_initial
    out = {"workload": "SIMPLE (SolverSIMPLE) on jittered triangle channels 2 x 1, inlet / "
                       "outlet / walls, the reference's split initial field, DT = 1/4000, "
                       "5 SIMPLE iterations per step, FP64 bit-exact",
           "unit": "time steps/s"}
    d = tempfile.mkdtemp(prefix="bench_simple_")
    for label, nx, ny, steps in (("sod_size", 95, 96, 40), ("large", 400, 300, 10)):
        path = os.path.join(d, label + ".msh")
        mg.write_msh(path, mg.reorient(mg.tri_box(nx, ny, 2.0, 1.0, jitter=0.2, seed=5,
                                                  left=mg.INLET, right=mg.OUTLET,
                                                  bottom=mg.WALL, top=mg.WALL),
                                       "random", seed=6))
        mesh = Mesh.read_msh(path)
        s = SimpleSolver(mesh)
        s.step(max(3, args.warmup))
        grp.barrier()
        t0 = time.perf_counter()
        s.step(steps)
        secs = grp.max(time.perf_counter() - t0)
        i = s.info()
        res = {"cells": mesh.n_cells, "faces": mesh.n_faces, "steps": steps,
               "value": round(steps * grp.ws / secs, 2), "ms_per_step": round(1e3 * secs / steps, 3),
               "gpu_launches": 1, "cluster_ctas": i.cluster, "threads_per_cta": i.threads,
               "gauss_seidel_levels": [i.momentum_levels, i.pressure_levels]}
        s.close()
        if not args.no_cpu and grp.ws == 1:
            from oracle import build as ob
            from oracle import pyoracle as po
            ob.build_oracle()
            om = po.read_msh(path)
            p0, f0 = reference_initial(mesh)
            n_cpu = 2 if mesh.n_cells < 100000 else 1
            t1 = time.perf_counter()
            po.simple_step(om, p0, f0, n_cpu)
            cs = time.perf_counter() - t1
            res["cpu_baseline"] = {"value": round(n_cpu / cs, 3), "unit": "time steps/s",
                                   "cores": 1, "kind": "port",
                                   "sample": f"{n_cpu} step(s) of the same mesh ({cs:.2f} s)"}
        out[label] = res
    # several independent cases in one launch, one thread-block cluster each
    from mstcfd.psolver import step_batch
    n_cases, steps = 8, 20
    solvers = []
    for k in range(n_cases):
        path = os.path.join(d, f"case{k}.msh")
        mg.write_msh(path, mg.reorient(mg.tri_box(95, 96, 2.0, 1.0, jitter=0.2, seed=30 + k,
                                                  left=mg.INLET, right=mg.OUTLET,
                                                  bottom=mg.WALL, top=mg.WALL),
                                       "random", seed=60 + k))
        solvers.append(SimpleSolver(Mesh.read_msh(path)))
    step_batch(solvers, 2)
    grp.barrier()
    t0 = time.perf_counter()
    step_batch(solvers, steps)
    secs = grp.max(time.perf_counter() - t0)
    out["batch"] = {"cases": n_cases, "cells_per_case": solvers[0].n_cells, "steps": steps,
                    "value": round(n_cases * steps * grp.ws / secs, 2),
                    "unit": "case time steps/s", "ms_per_batch_step": round(1e3 * secs / steps, 3),
                    "gpu_launches": 1, "cluster_ctas": solvers[0].info().batch_cluster,
                    "note": "mst_simple_step_batch: one cluster per case"}
    for s_ in solvers:
        s_.close()
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=40)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="mstcfd", choices=["mstcfd", "reference"])
    ap.add_argument("--n", type=int, default=1000, help="lattice size (n*n*2 cells)")
    ap.add_argument("--cpu-steps", type=int, default=3)
    ap.add_argument("--no-cpu", action="store_true",
                    help="skip the CPU-baseline sample (profiler runs)")
    ap.add_argument("--batch-cases", type=int, default=16,
                    help="cases of the batched wedge solve (0: skip)")
    ap.add_argument("--batch-cells", type=int, nargs=2, default=[20000, 60000])
    ap.add_argument("--batch-iters", type=int, default=20000)
    ap.add_argument("--warm-train", type=int, default=256,
                    help="training cases of the learned warm start (0: no warm start)")
    ap.add_argument("--warm-steps", type=int, default=2000)
    ap.add_argument("--fp32-until", type=float, default=1e-5,
                    help="the batch's production runs use the FP32 residual until this L2")
    ap.add_argument("--fp32-window", type=int, default=1000,
                    help="iterations of the FP32-phase stagnation / wait tests")
    ap.add_argument("--scale-cases", type=int, default=0,
                    help="cases of the batch-throughput line at scale (0: skip)")
    ap.add_argument("--scale-cells", type=int, nargs=2, default=[20000, 400000])
    ap.add_argument("--scale-iters", type=int, default=200)
    ap.add_argument("--tgv-n", type=int, default=128,
                    help="hexahedra per side of the 3D Taylor-Green mesh (x6 cells; 0: skip)")
    ap.add_argument("--tgv-steps", type=int, default=10)
    ap.add_argument("--network-only", action="store_true",
                    help="time only the network's GEMMs at batch scale (profiling)")
    ap.add_argument("--no-simple", action="store_true",
                    help="skip the pressure-based SIMPLE sub-line")
    args = ap.parse_args()
    ws, rank, local = _dist()
    workload = (f"isentropic vortex, periodic jittered Delaunay {args.n}x{args.n} "
                f"lattice ({2 * args.n * args.n} triangles), AUSM+ + van Leer, "
                f"RK2, CFL 0.5")
    config = {"workload": workload, "cells": 2 * args.n * args.n,
              "faces": 3 * args.n * args.n, "step": "one RK2 time step = 2 cell-updates per cell",
              "l2": "inputs larger than L2 (state + mesh ~0.5 GB)",
              "parallelism": f"replicas x{ws}"}
    if args.impl == "reference":
        if rank != 0:
            return
        from oracle import build as ob
        ob.build_oracle()
        m = _workload(args.n)
        from oracle import pyoracle as po  # noqa: F401
        # warmup steps then timed steps, each one RK2 step of the full mesh,
        # bounded to a few minutes in total
        run_cpu_sample(m, max(1, args.warmup), budget_s=20.0)
        v, cores, done, secs = run_cpu_sample(m, args.steps, budget_s=120.0)
        line = {"metric": METRIC, "value": round(v, 3), "unit": UNIT, "impl": "reference",
                "n_gpus": args.gpus, "steps": done, "warmup": args.warmup,
                "ms_per_step": round(1e3 * secs / done, 3), "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": config,
                "cpu_baseline": {"value": round(v, 3), "unit": UNIT, "cores": cores,
                                 "kind": "port",
                                 "sample": f"{done} RK2 steps of the full mesh"},
                "e2e": {"value": round(v, 3), "unit": UNIT, "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return
    grp = _Group(ws)
    if args.network_only:
        # the learned initial field's tensor-core GEMMs alone, at batch scale
        # (one forward + backward over the batch's cells, untrained weights)
        print(json.dumps({"network_gemm": run_network_only(args)}))
        return
    results, roof, nC = run_gpu(args, ws, rank, local, grp)
    batch_line = run_batch(args, ws, rank, grp) if args.batch_cases > 0 else None
    tgv_line = run_tgv3d(args, grp) if args.tgv_n > 0 else None
    scale_line = run_batch_scale(args, grp) if args.scale_cases > 0 else None
    simple_line = None if args.no_simple else run_simple(args, grp)
    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu:
        m = _workload(args.n)
        v, cores, done, secs = run_cpu_sample(m, args.cpu_steps, budget_s=25.0)
        cpu = {"value": round(v, 3), "unit": UNIT, "cores": cores, "kind": "port",
               "sample": f"{done} RK2 step(s) of the full {m['n_cells']}-cell mesh "
                         f"({secs:.1f} s, FP64, OpenMP)"}
    if rank != 0:
        return
    fp32, fp64 = results["fp32"], results["fp64"]
    line = {"metric": METRIC, "value": round(fp32["value"], 2), "unit": UNIT,
            "n_gpus": ws, "steps": fp32["steps"], "warmup": args.warmup,
            "ms_per_step": round(fp32["ms_per_step"], 5), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 flux / float-pair accumulate",
            "data": "synthetic", "config": config,
            "fp64": {"value": round(fp64["value"], 2), "unit": UNIT,
                     "ms_per_step": round(fp64["ms_per_step"], 5), "dtype": "f64",
                     "roofline": fp64.get("roofline"), "roofline_hbm": fp64.get("roofline_hbm")},
            "e2e": {k: (round(v, 2) if isinstance(v, float) else v)
                    for k, v in results["e2e"].items()},
            "gpu_launches": fp32["launches"],
            "roofline": roof, "cpu_baseline": cpu, "clocks": results.get("clocks"),
            "batch": batch_line, "tgv3d": tgv_line, "simple": simple_line}
    if scale_line:
        line["batch_scale"] = scale_line
    print(json.dumps(line))


if __name__ == "__main__":
    main()
