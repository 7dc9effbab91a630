"""CPU: the oracle against the reference's own LM driver.

The reference's src/lm.cu is compiled UNMODIFIED against the in-repo Eigen
stand-in (oracle/eigen_shim) and its host LM driver runs on the CPU, with its
three kernels restated in the CUDA-runtime stand-in (oracle/ref_host_runtime.cpp).
Where the reference checkout is present these tests build and run it live;
everywhere they check the committed full-precision runs
(tests/golden/reference_runs.json) against the oracle restatement.
"""
import json
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN

RUNS = json.loads((GOLDEN / "reference_runs.json").read_text())


def _ref_lm(oracle):
    try:
        return oracle.ReferenceLM()
    except FileNotFoundError:
        pytest.skip("reference checkout unavailable: the reference LM driver is not built")


def _traj_close(a, b, initial, rtol=1e-9):
    a, b = np.asarray(a), np.asarray(b)
    assert a.shape == b.shape
    return float(np.max(np.abs(a - b) / (np.abs(b) + 1e-12 * initial / rtol)))


def test_reference_lm_driver_matches_oracle_workload1(gba, oracle):
    """Live: the reference driver and the restatement on workload 1, 20 iterations."""
    ref = _ref_lm(oracle)
    prob = gba.synthetic(1)
    r, rc, rp = ref.solve(prob, max_iterations=20)
    o, oc, op = oracle.solve(prob, max_iterations=20, threads=2)
    assert r["termination"] == o["termination"] == "CONVERGENCE"
    assert r["iterations"] == o["iterations"]
    assert r["anomalies"] == 0
    assert _traj_close(o["trajectory"], r["trajectory"], r["initial_cost"]) < 1e-9
    assert np.max(np.abs(oc - rc)) <= 1e-7 * np.max(np.abs(rc))
    # and the committed run is this run
    e = RUNS["w1"]["reference"]
    assert _traj_close(r["trajectory"], e["trajectory"], e["initial_cost"]) < 1e-12


def test_reference_launch_bounds_test_passes():
    """The reference's own tests/test_launch_bounds.cpp, unmodified, on the reference driver."""
    import build_oracle

    if build_oracle.build_reference_lm() is None or not build_oracle.REF_LB_EXE.exists():
        pytest.skip("reference checkout unavailable")
    r = subprocess.run([str(build_oracle.REF_LB_EXE)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    assert "PASS" in r.stderr + r.stdout


def test_reference_driver_reports_failure_on_optimum(gba, oracle):
    """Zero-noise optimum: the reference driver and the restatement both end in
    FAILURE (every trial rejected) or CONVERGENCE, identically."""
    ref = _ref_lm(oracle)
    prob, truth = gba.synthetic(1, with_truth=True)
    zero = truth.copy()
    for e in range(zero.num_observations):
        c, q = zero.obs_camera[e], zero.obs_point[e]
        zero.obs_pixel[2 * e:2 * e + 2] = gba.snavely_residual(zero.cameras[9 * c:9 * c + 9],
                                                               zero.points[3 * q:3 * q + 3], np.zeros(2))
    r, _, _ = ref.solve(zero, max_iterations=5, max_inner_trials=4)
    o, _, _ = oracle.solve(zero, max_iterations=5, max_inner_trials=4, threads=2)
    assert r["termination"] == o["termination"]
    assert r["iterations"] == o["iterations"]


@pytest.mark.parametrize("name", sorted(RUNS))
def test_committed_runs_oracle_agrees_with_reference(name):
    """Every committed configuration: the restatement's trajectory within 1e-9
    of the reference driver's, same iterations and termination."""
    e = RUNS[name]
    if "oracle" not in e:
        pytest.skip("no restatement run recorded")
    r, o = e["reference"], e["oracle"]
    assert r["termination"] == o["termination"]
    assert r["iterations"] == o["iterations"]
    assert r["anomalies"] == o["anomalies"] == 0
    assert _traj_close(o["trajectory"], r["trajectory"], r["initial_cost"]) < 1e-9


def test_oracle_reproduces_committed_reference_run_workload1(gba, oracle):
    """Without the reference checkout: the restatement on this machine against
    the committed reference-driver run of workload 1."""
    e = RUNS["w1"]
    prob = gba.synthetic(1)
    import hashlib

    h = hashlib.sha256()
    for a in prob.arrays():
        h.update(a.tobytes())
    assert h.hexdigest() == e["fingerprint"]
    o, _, _ = oracle.solve(prob, max_iterations=e["max_iterations"], threads=2)
    assert _traj_close(o["trajectory"], e["reference"]["trajectory"], e["reference"]["initial_cost"]) < 1e-9


@pytest.mark.parametrize("workload,seed", [(1, 1), (2, 2), (4, 4)])
def test_oracle_generator_bit_identical_to_product(gba, oracle, workload, seed):
    """The CPU benchmark arm generates its problems with the oracle's own
    generator (nothing of the product loaded): same bits as the product's."""
    a, b = gba.synthetic(workload, seed), oracle.synthetic(workload, seed)
    for x, y in zip(a.arrays(), b.arrays()):
        assert x.dtype == y.dtype and np.array_equal(x, y)
