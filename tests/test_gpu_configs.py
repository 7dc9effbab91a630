"""GPU parity at the seeded workload configurations, through the C ABI.

The reference points are the REFERENCE's own LM driver (src/lm.cu compiled
unmodified against the Eigen stand-in and run on the CPU by the CUDA-runtime
stand-in, oracle/_ref) and the oracle restatement, recorded at full precision
in tests/golden/reference_runs.json by tests/golden/make_reference_runs.py:

  w1  16 / 22,000 / ~84k           plain, 20 iterations
  w2  257 / 65,000 / ~225k         plain, 30 iterations (dense S 2,313^2 on the device)
  w3  1,000 / 200,000 / ~800k      plain, 40 iterations (dense S 9,000^2) and the mixed form with
                                   FP64 refinement to 1e-8 (PCG tolerance 1e-4), up to 40 iterations
  w4  workload 3's shape, seed 4   plain, 40 iterations
  lb  the launch-bounds problem    plain (reference tests/test_launch_bounds.cpp)

Tolerances: the plain form's per-iteration cost 1e-9 relative to the
reference driver's (plus 1e-12 of the initial cost, for the launch-bounds
problem whose cost ends at round-off level); same iteration count and
termination; the mixed form's final cost within 0.1% of the reference's and
of the plain form's, with every refined Schur step at relative residual
<= 1e-8.
"""
import hashlib
import json

import numpy as np
import pytest

from conftest import GOLDEN, implicit_system

pytestmark = pytest.mark.gpu

RUNS = json.loads((GOLDEN / "reference_runs.json").read_text())


def _problem(gba, name):
    e = RUNS[name]
    prob = gba.launch_bounds_problem() if e["workload"] is None else gba.synthetic(e["workload"], e["seed"])
    h = hashlib.sha256()
    for a in prob.arrays():
        h.update(a.tobytes())
    if h.hexdigest() != e["fingerprint"]:
        pytest.fail(f"{name}: the generator produced a different problem on this machine than the one the "
                    "reference run used (fingerprint mismatch)")
    return prob, e


def _assert_trajectory(res, ref, rtol=1e-9):
    t_dev, t_ref = np.array(res.trajectory), np.array(ref["trajectory"])
    assert res.termination == ref["termination"]
    assert res.iterations == ref["iterations"]
    assert t_dev.shape == t_ref.shape
    floor = 1e-12 * ref["initial_cost"]
    worst = np.max(np.abs(t_dev - t_ref) / (np.abs(t_ref) + floor / rtol))
    assert worst <= rtol, worst


@pytest.mark.parametrize("name", [n for n in ("w1", "w2", "lb", "w3", "w4") if n in RUNS])
def test_plain_trajectory_matches_reference_driver(gba, name):
    prob, e = _problem(gba, name)
    ref = e["reference"]
    reader = gba.total_squared_error(prob) / 2
    res = gba.solve(prob.copy(), max_iterations=e["max_iterations"])
    assert abs(res.initial_cost - reader) <= 1e-9 * max(1.0, reader)
    assert res.anomalies == 0 and ref["anomalies"] == 0
    _assert_trajectory(res, ref)
    if "oracle" in e:  # the restatement agrees with the reference driver too
        _assert_trajectory(res, e["oracle"])


@pytest.mark.skipif("w3" not in RUNS, reason="workload 3 reference run not recorded")
def test_mixed_workload3_refined_to_1e8_reaches_reference_cost(gba):
    prob, e = _problem(gba, "w3")
    ref_final = e["reference"]["final_cost"]
    res = gba.solve(prob.copy(), max_iterations=40, form="mixed", refine_tol=1e-8, pcg_tol=1e-4)
    assert res.anomalies == 0
    assert abs(res.initial_cost - e["reference"]["initial_cost"]) <= 1e-9 * e["reference"]["initial_cost"]
    assert 0.0 < res.max_refine_residual <= 1e-8, res.max_refine_residual
    assert res.final_cost <= ref_final * (1 + 1e-3)
    plain = gba.solve(prob.copy(), max_iterations=40)
    assert res.final_cost <= plain.final_cost * (1 + 1e-3)
    print(f"w3: mixed final {res.final_cost:.12g} ({res.iterations} it, {res.pcg_iterations} PCG, "
          f"max refined residual {res.max_refine_residual:.2e}); reference {ref_final:.12g}; "
          f"plain {plain.final_cost:.12g}")


@pytest.mark.skipif("w3" not in RUNS, reason="workload 3 reference run not recorded")
def test_mixed_workload3_first_step_true_residual(gba):
    """The refined step of the first trial, checked in numpy FP64 on the
    system the refinement solves (FP32 Jacobian records, FP64 U, V, b)."""
    prob, _ = _problem(gba, "w3")
    lam = 1e-3
    with gba.Solver(prob, "mixed") as s:
        s.accumulate()
        assert s.damp_invert_v(lam) == 0
        iters, steps, relres = s.schur_pcg(lam, refine_tol=1e-8, pcg_tol=1e-4, pcg_max_iters=200)
        dc = s.download("dc")
        rhs, matvec = implicit_system(s, prob, lam)
    true_rel = np.linalg.norm(rhs - matvec(dc)) / np.linalg.norm(rhs)
    assert relres <= 1e-8
    assert true_rel <= 1.01e-8, (true_rel, relres)
    assert abs(true_rel - relres) <= 1e-10
