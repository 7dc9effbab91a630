"""Generates tests/golden/reference_runs.json: cost trajectories of the
REFERENCE's own LM driver (src/lm.cu, compiled unmodified against the Eigen
stand-in and run on the CPU by the CUDA-runtime stand-in, oracle/_ref) and of
the oracle's restatement (oracle/lm_oracle.cpp) on the seeded workloads:

  w1  16 / 22,000 / ~84k         20 iterations
  w2  257 / 65,000 / ~225k       30 iterations
  w3  1,000 / 200,000 / ~800k    40 iterations
  w4  workload 3's shape, seed 4 40 iterations
  lb  the launch-bounds problem (C 8, P 400,000, E 800,000; reference tests/test_launch_bounds.cpp)

Each entry also holds a SHA-256 fingerprint of the problem arrays, so that a
test on another machine can check that the library's generator produced the
same problem before comparing trajectories. Needs the reference checkout (see
oracle/build_oracle.py); no GPU:

    python tests/golden/make_reference_runs.py [--only w1,w2,lb] [--threads N]

Entries are merged into the existing file.
"""
from __future__ import annotations

import argparse
import hashlib
import json
import os
import sys
import time
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path[:0] = [str(ROOT / "gpu-bundle-adjustment_gb300"), str(ROOT / "oracle")]

OUT = HERE / "reference_runs.json"
CASES = {"w1": (1, 1, 20), "w2": (2, 2, 30), "w3": (3, 3, 40), "w4": (3, 4, 40), "lb": (None, None, 50)}


def fingerprint(prob) -> str:
    h = hashlib.sha256()
    for a in prob.arrays():
        h.update(a.tobytes())
    return h.hexdigest()


def make_problem(name):
    import gba_gb300 as gba

    workload, seed, _ = CASES[name]
    return gba.launch_bounds_problem() if workload is None else gba.synthetic(workload, seed)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--only", default=",".join(CASES))
    ap.add_argument("--threads", type=int, default=0)
    ap.add_argument("--no-oracle", action="store_true", help="skip the restatement's run (reference driver only)")
    args = ap.parse_args()
    if args.threads:
        os.environ["GBA_SHIM_THREADS"] = str(args.threads)
    import numpy as np

    import oracle

    ref = oracle.ReferenceLM()
    data = json.loads(OUT.read_text()) if OUT.exists() else {}
    for name in args.only.split(","):
        workload, seed, iters = CASES[name]
        prob = make_problem(name)
        t0 = time.perf_counter()
        r, _, _ = ref.solve(prob, max_iterations=iters)
        t_ref = time.perf_counter() - t0
        entry = {
            "workload": workload, "seed": seed, "max_iterations": iters,
            "cameras": prob.num_cameras, "points": prob.num_points, "observations": prob.num_observations,
            "fingerprint": fingerprint(prob),
            "reference": {k: r[k] for k in ("initial_cost", "final_cost", "iterations", "termination", "anomalies",
                                            "trials", "trajectory")},
            "reference_seconds": t_ref,
        }
        if not args.no_oracle:
            t0 = time.perf_counter()
            o, _, _ = oracle.solve(prob, max_iterations=iters, threads=args.threads)
            t_or = time.perf_counter() - t0
            entry["oracle"] = {k: o[k] for k in ("initial_cost", "final_cost", "iterations", "termination",
                                                 "anomalies", "trajectory")}
            entry["oracle_seconds"] = t_or
            a, b = np.array(r["trajectory"]), np.array(o["trajectory"])
            entry["oracle_vs_reference_max_rel"] = (float(np.max(np.abs(a - b) / np.abs(a)))
                                                     if a.shape == b.shape else None)
        data[name] = entry
        OUT.write_text(json.dumps(data, indent=1) + "\n")
        print(name, prob.num_cameras, prob.num_points, prob.num_observations, r["iterations"], r["termination"],
              f"final {r['final_cost']:.17g}", f"{t_ref:.1f} s", entry.get("oracle_vs_reference_max_rel"),
              flush=True)


if __name__ == "__main__":
    main()
