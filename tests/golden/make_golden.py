"""Generates the committed golden fixtures of this directory.

Run where the reference checkout is available (it compiles the reference's own
src/bal_reader.cpp through oracle/build_oracle.py and records its outputs):

    python tests/golden/make_golden.py

Outputs (small, committed):
  residual_golden.json  BAL-like edges (including |rodrigues| below the 1e-12 /
                        1e-24 branch thresholds) and the reference
                        snavely_residual of each, %.17g.
  fd_cases.json         the two finite-difference Jacobian cases of the
                        reference test (tests/test_vs_ceres.cpp:34-39).
  tiny_problem.txt      a 5-camera / 300-point synthetic BAL file (written by
                        this library's writer) and tiny_problem.json with the
                        reference reader's dimensions and total squared error.
"""
from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT / "oracle"))
sys.path.insert(0, str(ROOT / "gpu-bundle-adjustment_gb300"))


def main() -> None:
    import oracle  # noqa: E402

    ref = oracle.ReferenceReader()
    rng = np.random.default_rng(20261203)
    edges = []
    for i in range(200):
        cam = np.concatenate([
            rng.normal(0, 0.3, 3), rng.normal(0, 1, 3), [rng.uniform(300, 700)], rng.normal(0, 0.05, 1),
            rng.normal(0, 0.005, 1)
        ])
        if i % 20 == 0:
            cam[:3] = rng.normal(0, 1e-13, 3)  # below the CPU 1e-12 branch threshold
        elif i % 20 == 1:
            cam[:3] = rng.normal(0, 1e-9, 3)  # tiny but on the Rodrigues branch
        elif i % 20 == 2:
            cam[:3] = 0.0
        pt = np.array([rng.uniform(-3, 3), rng.uniform(-3, 3), rng.uniform(-12, -3)])
        obs = rng.normal(0, 300, 2)
        r = ref.snavely_residual(cam, pt, obs)
        edges.append(dict(cam=cam.tolist(), pt=pt.tolist(), obs=obs.tolist(), residual=r.tolist()))
    (HERE / "residual_golden.json").write_text(json.dumps(dict(
        source="reference src/bal_reader.cpp snavely_residual, compiled from source", edges=edges), indent=1))

    cases = [
        [0.1, -0.5, 0.3, 0.02, 0.01, -1.0, 500.0, -0.2, 0.01, 1.0, 2.0, 30.0, 100.0, -80.0],
        [1e-8, 2e-8, -1e-8, -0.05, 0.2, 0.4, 350.0, 0.1, -0.001, -2.0, 1.0, 25.0, -250.0, 300.0],
    ]
    (HERE / "fd_cases.json").write_text(json.dumps(dict(
        source="reference tests/test_vs_ceres.cpp:34-39 (camera[9], point[3], pixel[2])", cases=cases,
        eps=1e-6, tolerance=1e-5), indent=1))

    import gba_gb300 as gba  # noqa: E402

    path = HERE / "tiny_problem.txt"
    h = gba.C.c_void_p()
    gba._check(gba.lib.gba_host_problem_synthetic_custom(5, 300, 2, 5, 1.5, 0.0, 0.0, 11, gba.C.byref(h)))
    gba._check(gba.lib.gba_host_problem_save(h, str(path).encode()))
    gba.lib.gba_host_problem_free(h)
    cams, pts, oc, op, px = ref.load_bal(path)
    sse = ref.lib.ref_total_squared_error(cams.size // 9, pts.size // 3, oc.size, oracle._d(cams), oracle._d(pts),
                                          oracle._i(oc), oracle._i(op), oracle._d(px))
    (HERE / "tiny_problem.json").write_text(json.dumps(dict(
        source="reference load_bal + total_squared_error on tiny_problem.txt", num_cameras=cams.size // 9,
        num_points=pts.size // 3, num_observations=int(oc.size), total_squared_error=sse), indent=1))
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main()
