"""Times the reference's own density path (compiled into oracle/_ref) beside
the oracle's C restatement (the port bench.py's CPU arms use) on the same
first-order workload, the one the reference can run as shipped: AUSM+,
first order, explicit Euler at a fixed DT, on a jittered triangle box
written as a Fluent mesh.  Both use the same OpenMP thread count; both
compute the same states (the parity tests pin them bit for bit).

TEST INFRASTRUCTURE ONLY: needs the reference sources (oracle/build.py
REF_SRC); prints one JSON line.

    python -m oracle.calibrate_port [--nx 700] [--ny 350] [--steps 20]
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
for _p in (ROOT, os.path.join(ROOT, "mst-cfd_gb300")):
    if _p not in sys.path:
        sys.path.insert(0, _p)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--nx", type=int, default=700)
    ap.add_argument("--ny", type=int, default=350)
    ap.add_argument("--steps", type=int, default=20)
    args = ap.parse_args()
    from mstcfd import meshgen as mg
    from oracle import build, pyoracle as po
    if not build.build_ref():
        raise SystemExit("reference sources not available")
    build.build_oracle()
    m = mg.tri_box(args.nx, args.ny, 4.0, 2.0, jitter=0.2, seed=3)
    d = tempfile.mkdtemp(prefix="mstcal_")
    path = os.path.join(d, "box.msh")
    mg.write_msh(path, m)
    threads = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    exe = os.path.join(build.REF_OUT, "ref_rho_ausm_o1")
    r = subprocess.run([exe, path, d, "--bench", str(args.steps)], check=True,
                       capture_output=True, text=True)
    line = [ln for ln in r.stdout.splitlines() if ln.startswith("BENCH")][-1]
    ref = {k: float(v) for k, v in (kv.split("=") for kv in line.split()[1:])}
    om = po.read_msh(path)
    # the reference's own initial field (Time.cpp:26-36): Sod split at x = 0.5
    left = om.cell_ctr[:, 0] <= 0.5
    q = mg.primitive_to_q(np.where(left, 1.0, 0.125), np.zeros(om.n_cells),
                          np.zeros(om.n_cells), np.where(left, 1.0, 0.1))
    prm = po.params_ext(0, 1)
    q, _ = po.step_ext(om, prm, q, 1)  # warm-up, as the reference harness does
    t0 = time.perf_counter()
    po.step_ext(om, prm, q, args.steps)
    sec = time.perf_counter() - t0
    port = om.n_cells * args.steps / sec / 1e6
    print(json.dumps({"workload": f"AUSM+ first order, explicit Euler, fixed DT, "
                                  f"{om.n_cells}-triangle box", "steps": args.steps,
                      "threads_port": threads, "threads_reference": int(ref["threads"]),
                      "reference_mcups": round(ref["mcups"], 3), "port_mcups": round(port, 3),
                      "port_over_reference": round(port / ref["mcups"], 3),
                      "cpu": os.uname().machine}))


if __name__ == "__main__":
    main()
