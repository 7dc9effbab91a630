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


MODEL = GOLDEN.parents[1] / "gpu-bundle-adjustment_gb300" / "models" / "coarse_mlp.bin"


@pytest.mark.skipif(not MODEL.exists() or "w4" not in RUNS, reason="trained model or workload 4 run missing")
def test_learned_vs_block_jacobi_vs_exact_workload4(gba):
    """Workload 4 (workload 3's shape, seed 4): the learned coarse correction
    against block-Jacobi alone and the exact dense step, on the same trial
    (lambda 1e-3 at the initial parameters) and over whole solves.
      - inner PCG iterations of the step refined to 1e-8 (PCG tolerance 1e-4):
        the learned form needs at most 80% of block-Jacobi's;
      - S-norm step error ||dc - dc*||_S / ||dc*||_S after 10 PCG iterations
        (dc* the plain form's exact FP64 step, S its dense FP64 system): the
        learned one is smaller; refined, both reach the FP32-Jacobian floor;
      - whole LM solves at the strict targets: the learned form's PCG work is at
        most 80% of block-Jacobi's and both final costs are within 0.1% of the
        reference driver's."""
    prob, e = _problem(gba, "w4")
    lam = 1e-3
    C = prob.num_cameras
    with gba.Solver(prob, "plain") as s:
        s.set_schur_layout("dense")
        s.accumulate()
        assert s.damp_invert_v(lam) == 0
        assert s.schur_dense(lam) == 0
        _, _, _, n_pad = s.dims()
        L = np.tril(s.download("S").reshape(n_pad, n_pad).T[:9 * C, :9 * C])
        dc_exact = s.download("dc")

    def snorm(x):
        y = L.T @ x
        return float(np.sqrt(y @ y))

    ref_norm = snorm(dc_exact)
    out = {}
    for mode in ("block-jacobi", "learned"):
        with gba.Solver(prob, "learned") as s:
            s.load_model(MODEL)
            s.set_preconditioner(mode)
            s.accumulate()
            assert s.damp_invert_v(lam) == 0
            iters, _, relres = s.schur_pcg(lam, learned=True, refine_tol=1e-8, pcg_tol=1e-4, pcg_max_iters=500)
            dc = s.download("dc")
            s.schur_pcg(lam, learned=True, refine_tol=1e-30, refine_max_steps=1, pcg_tol=0.0, pcg_max_iters=10)
            dc10 = s.download("dc")
        out[mode] = dict(iters=iters, relres=relres, err=snorm(dc - dc_exact) / ref_norm,
                         err10=snorm(dc10 - dc_exact) / ref_norm)
    bj, le = out["block-jacobi"], out["learned"]
    print(f"w4 one trial: {out}")
    assert bj["relres"] <= 1e-8 and le["relres"] <= 1e-8
    assert le["iters"] <= 0.8 * bj["iters"], out
    assert le["err10"] < bj["err10"], out
    assert max(bj["err"], le["err"]) < 1e-3, out
    strict = dict(refine_tol=1e-8, pcg_tol=1e-4, max_iterations=40)
    ref_final = e["reference"]["final_cost"]
    r_bj = gba.solve(prob.copy(), form="mixed", **strict)
    r_le = gba.solve(prob.copy(), form="learned", model_path=str(MODEL), **strict)
    print(f"w4 solves: block-Jacobi {r_bj.pcg_iterations} PCG / {r_bj.final_cost:.12g}; learned "
          f"{r_le.pcg_iterations} PCG / {r_le.final_cost:.12g} (choice {r_le.learned_choice}); "
          f"reference {ref_final:.12g}")
    assert r_le.learned_choice == 1
    assert r_le.pcg_iterations <= 0.8 * r_bj.pcg_iterations
    for r in (r_bj, r_le):
        assert r.anomalies == 0 and r.final_cost <= ref_final * (1 + 1e-3)
        assert r.max_refine_residual <= 1e-8
