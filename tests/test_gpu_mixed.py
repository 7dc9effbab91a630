"""GPU: the mixed-precision form (FP32 Jacobians with FP64 accumulation,
implicit FP32 Schur matvecs in block-Jacobi PCG, iterative refinement with a
float-float residual, float-float cost).

Gates: normal equations within FP32 rounding of the FP64 oracle; the refined
Schur step satisfies the FP64 residual target 1e-8 and agrees with the exact
(plain, dense) step; the LM solve reaches the FP64 oracle's final cost within
0.1% (the spec accuracy bar), with FP64 cost evaluation (initial cost =
reader cost to 1e-9).
"""
import numpy as np
import pytest

from conftest import jacobian_rows, implicit_system, rel_err

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def small(gba):
    return gba.synthetic_custom(9, 1500, 2, 7, 1.4, seed=31)


def test_mixed_normal_equations_within_fp32(gba, oracle, small):
    with gba.Solver(small, "mixed") as s:
        sse = s.accumulate()
        U = s.download("U").reshape(-1, 9, 9)
        bc = s.download("bc")
        Vp = s.download("V").reshape(-1, 6)
        bp = s.download("bp")
        J = jacobian_rows(s)
        order = s.download("order")
    ref = oracle.accumulate(small)
    # the cost is float-float (~48-bit significands); the residual cancels
    # ~500 px predictions against the observations, so 1e-11 bounds it
    assert abs(sse - ref["sse"]) <= 1e-11 * ref["sse"]
    assert rel_err(U, ref["U"]) < 2e-5
    assert rel_err(bc, ref["bc"]) < 2e-5
    assert rel_err(Vp[:, 0], ref["V"][:, 0, 0]) < 2e-5
    assert rel_err(bp, ref["bp"]) < 2e-5
    # Jacobian records in slot order -> W = Jc^T Jp per observation
    Jc = J[:, :18].reshape(-1, 2, 9).astype(np.float64)
    Jp = J[:, 18:].reshape(-1, 2, 3).astype(np.float64)
    W = np.einsum("eri,erj->eij", Jc, Jp)
    assert rel_err(W, ref["W"][order]) < 2e-5


def test_refined_step_matches_exact_dense_step(gba, oracle, small):
    lam = 1e-3
    ref = oracle.schur_step(small, lam, threads=4)
    assert ref["status"] == 0
    with gba.Solver(small, "mixed") as s:
        s.accumulate()
        assert s.damp_invert_v(lam) == 0
        iters, steps, relres = s.schur_pcg(lam, refine_tol=1e-8, pcg_tol=1e-2, pcg_max_iters=500)
        dc = s.download("dc")
        denom = s.back_substitute(lam)
        dp = s.download("dp")
    assert relres <= 1e-8, relres
    assert steps >= 1 and iters >= 1
    # the refined system is the one with FP32-rounded Jacobians: agreement to
    # FP32 rounding amplified by the conditioning of S
    assert rel_err(dc, ref["dc"]) < 1e-3
    assert rel_err(dp, ref["dp"]) < 1e-3
    assert abs(denom - ref["denom"]) < 1e-3 * abs(ref["denom"])


def test_pcg_deterministic(gba, small):
    """The ordered two-pass product: bit-identical reruns."""
    lam = 1e-2
    out = []
    for _ in range(2):
        with gba.Solver(small, "mixed") as s:
            assert not s.set_matvec("two-pass")
            s.accumulate()
            s.damp_invert_v(lam)
            s.schur_pcg(lam, refine_tol=1e-8)
            out.append(s.download("dc"))
    assert np.array_equal(out[0], out[1])


def test_lm_trial_reuses_the_refinement_back_substitution(gba, small):
    """The LM driver's trial skips the back-substitution's point pass when the
    last refinement check already ran it at the same dc. The trial is the same
    as the stage functions' (which always recompute it): bit-identical trial
    parameters and cost, in the deterministic two-pass product."""
    lam = 1e-3
    opts = dict(refine_tol=1e-10, pcg_tol=1e-3, pcg_max_iters=500, refine_max_steps=12)
    with gba.Solver(small, "mixed") as s:
        res = s.run(max_iterations=1, initial_lambda=lam, deterministic=1, **opts)
        cams_lm, pts_lm = s.get_params()
    assert res.iterations == 1 and res.trials == 1  # the first trial was accepted
    assert res.refine_steps >= 2  # a later step's check ran the back-substitution
    with gba.Solver(small, "mixed") as s:
        assert not s.set_matvec("two-pass")
        s.accumulate()
        assert s.damp_invert_v(lam) == 0
        _, steps, relres = s.schur_pcg(lam, **opts)
        s.back_substitute(lam)
        trial = s.trial_cost()
        s.accept()
        cams, pts = s.get_params()
    assert steps == res.refine_steps and relres <= 1e-10
    assert np.array_equal(cams, cams_lm) and np.array_equal(pts, pts_lm)
    assert trial / 2.0 == res.final_cost  # trial_cost() is the SSE, final_cost SSE / 2


def test_mixed_lm_reaches_oracle_cost_workload1(gba, oracle):
    prob = gba.synthetic(1)
    ref, _, _ = oracle.solve(prob, max_iterations=20)
    reader = gba.total_squared_error(prob) / 2
    res = gba.solve(prob.copy(), max_iterations=20, form="mixed")
    assert abs(res.initial_cost - reader) <= 1e-9 * max(1.0, reader)
    assert res.anomalies == 0
    assert res.final_cost <= ref["final_cost"] * (1 + 1e-3)
    assert res.pcg_iterations > 0 and res.refine_steps > 0


def test_mixed_lm_launch_bounds(gba):
    prob = gba.launch_bounds_problem(400000)
    res = gba.solve(prob, form="mixed")
    assert res.initial_cost > 1.0
    assert res.anomalies == 0
    assert res.final_cost < 1e-4 * res.initial_cost


def test_mixed_huber_reaches_oracle_cost_workload1(gba, oracle):
    """Huber loss through the FP32 implicit-Schur path: final robust cost within 0.1% of the oracle's."""
    prob = gba.synthetic(1)
    ref, _, _ = oracle.solve(prob, max_iterations=15, huber_delta=1.0)
    res = gba.solve(prob.copy(), max_iterations=15, form="mixed", loss="huber", huber_delta=1.0)
    assert abs(res.initial_cost - ref["initial_cost"]) <= 1e-9 * ref["initial_cost"]
    assert res.anomalies == 0
    assert res.final_cost <= ref["final_cost"] * (1 + 1e-3)


def test_loose_target_fast_path(gba, small):
    """refine_tol >= 1e-3: FP32 right-hand side, the converged inner solve as its
    own check, FP32 back-substitution. The true residual of the step meets the
    target (up to FP32 rounding) and dp follows from dc."""
    lam = 1e-3
    with gba.Solver(small, "mixed") as s:
        s.accumulate()
        assert s.damp_invert_v(lam) == 0
        iters, steps, relres = s.schur_pcg(lam, refine_tol=0.1, pcg_tol=0.1, pcg_max_iters=500)
        dc = s.download("dc")
        s.back_substitute(lam)
        dp = s.download("dp")
        rhs, matvec = implicit_system(s, small, lam)
    assert steps == 1 and 1 <= iters and relres <= 0.1
    true_rel = np.linalg.norm(rhs - matvec(dc)) / np.linalg.norm(rhs)
    assert true_rel <= 0.1 + 1e-4, (true_rel, relres)
    assert abs(true_rel - relres) <= 1e-4
    assert rel_err(dp, matvec.point_step(dc)) < 1e-4  # FP32 products, bp - W^T dc cancels


def test_mixed_lm_loose_target_reaches_oracle_cost_workload1(gba, oracle):
    """Inexact steps (forcing 0.1): the LM solve still reaches the FP64 oracle's
    final cost within 0.1%."""
    prob = gba.synthetic(1)
    ref, _, _ = oracle.solve(prob, max_iterations=20)
    res = gba.solve(prob.copy(), max_iterations=20, form="mixed", refine_tol=0.1, pcg_tol=0.1)
    assert res.anomalies == 0
    assert res.final_cost <= ref["final_cost"] * (1 + 1e-3)


def test_float_float_refinement_residual_is_fp64_accurate(gba, small):
    """The right-hand side and the refinement residual are computed in float-float
    products with FP64 sums; checked here against numpy FP64 on the same system."""
    lam = 1e-3
    with gba.Solver(small, "mixed") as s:
        s.accumulate()
        assert s.damp_invert_v(lam) == 0
        iters, steps, relres = s.schur_pcg(lam, refine_tol=1e-10, pcg_tol=1e-3, pcg_max_iters=500)
        rhs_dev = s.download("rhs")[:9 * small.num_cameras]
        dc = s.download("dc")
        rhs, matvec = implicit_system(s, small, lam)
    assert rel_err(rhs_dev, rhs) < 1e-12
    r = rhs - matvec(dc)
    true_rel = np.linalg.norm(r) / np.linalg.norm(rhs)
    assert relres <= 1e-10, relres
    assert true_rel <= 2e-10, (true_rel, relres)


@pytest.mark.parametrize("delta", [0.0, 2.0])
def test_float_float_cost_matches_oracle(gba, oracle, small, delta):
    """Trial cost of the mixed form (float-float residual pass) against the FP64
    oracle at perturbed parameters, plain and Huber."""
    rng = np.random.default_rng(5)
    cams = small.cameras + rng.normal(0, 1e-3, small.cameras.shape)
    pts = small.points + rng.normal(0, 1e-2, small.points.shape)
    with gba.Solver(small, "mixed") as s:
        if delta > 0:
            s.set_loss("huber", delta)
        s.set_params(cams, pts)
        sse = s.accumulate()
    ref = oracle.cost(small, cams, pts, huber_delta=delta)
    assert abs(sse - ref) <= 1e-11 * ref


def _rodrigues(w):
    th = np.linalg.norm(w)
    k = w / th
    K = np.array([[0, -k[2], k[1]], [k[2], 0, -k[0]], [-k[1], k[0], 0]])
    return np.eye(3) * np.cos(th) + np.sin(th) * K + (1 - np.cos(th)) * np.outer(k, k)


def test_float_float_cost_falls_back_to_fp64_out_of_range(gba, oracle, small):
    """A point 1e-6 from a camera's plane: its residual (~1e28 px) leaves FP32's
    range in float-float; that slot is re-evaluated in FP64, so the cost stays
    finite and equal to the FP64 oracle's (no anomaly)."""
    cams, pts = small.cameras.copy(), small.points.copy()
    e = 0
    c, p = small.obs_camera[e], small.obs_point[e]
    R = _rodrigues(cams[9 * c:9 * c + 3])
    target = np.array([0.3, 0.2, -1e-6])
    pts[3 * p:3 * p + 3] = R.T @ (target - cams[9 * c + 3:9 * c + 6])
    ref = oracle.cost(small, cams, pts)
    assert np.isfinite(ref) and ref > 1e40
    with gba.Solver(small, "mixed") as s:
        s.set_params(cams, pts)
        sse = s.accumulate()
    assert np.isfinite(sse)
    assert abs(sse - ref) <= 1e-6 * ref


def test_mixed_normal_equations_first_order_rotation_branch(gba, oracle):
    """A camera with a zero rotation vector takes the first-order branch
    (R X = X + a x X, dRX/da = -[X]x): the per-camera precomputed records of the
    FP32 Jacobian pass reproduce it (U, bc, V, bp within FP32 rounding)."""
    prob = gba.synthetic_custom(5, 600, 2, 5, 1.4, seed=41)
    prob.cameras[9 * 2:9 * 2 + 3] = 0.0
    prob.cameras[9 * 3:9 * 3 + 3] = [1e-13, -2e-13, 0.0]
    with gba.Solver(prob, "mixed") as s:
        s.accumulate()
        U = s.download("U").reshape(-1, 9, 9)
        bc = s.download("bc")
        bp = s.download("bp")
    ref = oracle.accumulate(prob)
    assert rel_err(U, ref["U"]) < 2e-5
    assert rel_err(bc, ref["bc"]) < 2e-5
    assert rel_err(bp, ref["bp"]) < 2e-5


@pytest.fixture(scope="module")
def long_tracks(gba):
    """Every point observed ~300 times: point chunks with more slots than one
    CTA pass (256), the multi-pass paths of the point kernels."""
    return gba.synthetic_custom(320, 40, 290, 310, 1.2, seed=3)


@pytest.mark.parametrize("form", ["plain", "mixed"])
def test_long_tracks_normal_equations(gba, oracle, long_tracks, form):
    with gba.Solver(long_tracks, form) as s:
        sse = s.accumulate()
        V = s.download("V").reshape(-1, 6)
        bp = s.download("bp")
        bc = s.download("bc")
    ref = oracle.accumulate(long_tracks)
    tol = 1e-11 if form == "plain" else 2e-5
    assert abs(sse - ref["sse"]) <= 1e-11 * ref["sse"]
    assert rel_err(V[:, 0], ref["V"][:, 0, 0]) < tol
    assert rel_err(bp, ref["bp"]) < tol
    assert rel_err(bc, ref["bc"]) < tol


def test_long_tracks_refined_step(gba, oracle, long_tracks):
    """Schur step through the multi-pass point kernels: refined to 1e-10 and
    agreeing with the exact (numpy FP64) system of the FP32 Jacobians."""
    lam = 1e-3
    with gba.Solver(long_tracks, "mixed") as s:
        s.accumulate()
        assert s.damp_invert_v(lam) == 0
        _, _, relres = s.schur_pcg(lam, refine_tol=1e-10, pcg_tol=1e-3, pcg_max_iters=500)
        rhs_dev = s.download("rhs")[:9 * long_tracks.num_cameras]
        dc = s.download("dc")
        s.back_substitute(lam)
        dp = s.download("dp")
        rhs, matvec = implicit_system(s, long_tracks, lam)
    assert rel_err(rhs_dev, rhs) < 1e-12
    assert relres <= 1e-10
    assert np.linalg.norm(rhs - matvec(dc)) / np.linalg.norm(rhs) <= 2e-10
    assert rel_err(dp, matvec.point_step(dc)) < 1e-9


def test_repeated_solves_bit_identical_and_cache_release(gba):
    """Solves allocate from the device memory pool: repeated solves (reusing
    cached memory) and a solve after the cache is released give bit-identical
    results with the deterministic option (every reduction is ordered)."""
    prob = gba.synthetic_custom(9, 1500, 2, 7, 1.4, seed=31)
    runs = []
    for i in range(3):
        if i == 2:
            gba.release_cached_memory()
        run = prob.copy()
        r = gba.solve(run, max_iterations=6, form="mixed", refine_tol=0.1, pcg_tol=0.1, deterministic=1)
        runs.append((r.trajectory, run.cameras.copy(), run.points.copy()))
    for traj, cams, pts in runs[1:]:
        assert traj == runs[0][0]
        assert np.array_equal(cams, runs[0][1]) and np.array_equal(pts, runs[0][2])
