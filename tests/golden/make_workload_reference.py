"""Generates tests/golden/workload_reference.json: the FP64 reference final
cost of the benchmark workloads, i.e. the plain all-FP64 form's converged LM
cost (exact dense Schur solve, DMMA Cholesky).

The plain form is the FP64 oracle at these sizes: it follows the CPU oracle's
cost trajectory to 1e-9 on the workloads the CPU oracle can run
(tests/test_gpu_plain.py); the CPU oracle itself cannot factor the 45,000 x
45,000 system of workload 5 in reasonable time. Needs a GPU:

    python tests/golden/make_workload_reference.py [--workload 5] [--out PATH]

Entries are keyed "workload:seed" and merged into the existing file.
"""
from __future__ import annotations

import argparse
import json
import sys
import time
from pathlib import Path

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parents[1] / "gpu-bundle-adjustment_gb300"))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", type=int, default=5)
    ap.add_argument("--seed", type=int, default=None)
    ap.add_argument("--max-iterations", type=int, default=50)
    ap.add_argument("--out", default=str(HERE / "workload_reference.json"))
    args = ap.parse_args()
    seed = args.workload if args.seed is None else args.seed

    import build as gba_build

    gba_build.build()
    import gba_gb300 as gba

    prob = gba.synthetic(args.workload, seed)
    t0 = time.time()
    res = gba.solve(prob, form="plain", max_iterations=args.max_iterations)
    wall = time.time() - t0
    out = Path(args.out)
    data = json.loads(out.read_text()) if out.exists() else {}
    data[f"{args.workload}:{seed}"] = {
        "final_cost": res.final_cost,
        "initial_cost": res.initial_cost,
        "iterations": res.iterations,
        "trials": res.trials,
        "termination": res.termination,
        "anomalies": res.anomalies,
        "solve_seconds": res.total_time_s,
        "wall_seconds": wall,
        "phases": res.phases,
        "trajectory": res.trajectory,
        "trajectory_time_s": res.trajectory_time_s,
        "cameras": prob.num_cameras,
        "points": prob.num_points,
        "observations": prob.num_observations,
        "form": "plain (FP64, dense Schur, DMMA Cholesky)",
    }
    out.write_text(json.dumps(data, indent=1))
    print(json.dumps({k: v for k, v in data[f"{args.workload}:{seed}"].items() if not k.startswith("trajectory")}))


if __name__ == "__main__":
    main()
