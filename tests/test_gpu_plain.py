"""GPU parity of the plain (all-FP64) form against the oracle, through the C ABI.

Mirrors the reference tests: test_schur.cu (batched 9x9 / 3x3 to 1e-9),
test_vs_ceres.cpp gates (initial cost = reader cost to 1e-9, zero anomalies,
CONVERGENCE), test_launch_bounds.cpp (P = 400,000 > one launch's worth of
threads: final < 1e-4 initial). Tolerances: FP64 stage outputs 1e-9 relative
(different summation orders and device vs host libm), the per-iteration LM cost
trajectory 1e-9 relative.
"""
import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


@pytest.fixture(scope="module")
def small(gba):
    return gba.synthetic_custom(7, 900, 2, 6, 1.4, seed=21)


def test_eval_edges_f64_matches_oracle(gba, oracle, torch_cuda, small):
    torch = torch_cuda
    p = small
    E = p.num_observations
    cams, pts, oc, op, px = (_dev(torch, a) for a in p.arrays())
    r = torch.empty(2 * E, dtype=torch.float64, device="cuda")
    jc = torch.empty(18 * E, dtype=torch.float64, device="cuda")
    jp = torch.empty(6 * E, dtype=torch.float64, device="cuda")
    gba.eval_edges(64, cams.data_ptr(), pts.data_ptr(), oc.data_ptr(), op.data_ptr(), px.data_ptr(), E,
                   r.data_ptr(), jc.data_ptr(), jp.data_ptr())
    torch.cuda.synchronize()
    r, jc, jp = (t.cpu().numpy() for t in (r, jc, jp))
    worst = 0.0
    for e in range(0, E, 7):
        c, q = p.obs_camera[e], p.obs_point[e]
        r0, jc0, jp0 = oracle.residual_jacobian(p.cameras[9 * c:9 * c + 9], p.points[3 * q:3 * q + 3],
                                                p.obs_pixel[2 * e:2 * e + 2])
        for a, b in ((r[2 * e:2 * e + 2], r0), (jc[18 * e:18 * e + 18], jc0.ravel()), (jp[6 * e:6 * e + 6], jp0.ravel())):
            worst = max(worst, float(np.max(np.abs(a - b)) / max(1.0, np.max(np.abs(b)))))
    assert worst < 1e-9, worst


def test_eval_edges_f32_within_fp32_tolerance(gba, oracle, torch_cuda, small):
    torch = torch_cuda
    p = small
    E = p.num_observations
    cams, pts, oc, op, px = (_dev(torch, a) for a in p.arrays())
    r = torch.empty(2 * E, dtype=torch.float32, device="cuda")
    jc = torch.empty(18 * E, dtype=torch.float32, device="cuda")
    gba.eval_edges(32, cams.data_ptr(), pts.data_ptr(), oc.data_ptr(), op.data_ptr(), px.data_ptr(), E,
                   r.data_ptr(), jc.data_ptr(), 0)
    torch.cuda.synchronize()
    r, jc = r.cpu().numpy().astype(np.float64), jc.cpu().numpy().astype(np.float64)
    worst_r, worst_j = 0.0, 0.0
    for e in range(0, E, 11):
        c, q = p.obs_camera[e], p.obs_point[e]
        r0, jc0, _ = oracle.residual_jacobian(p.cameras[9 * c:9 * c + 9], p.points[3 * q:3 * q + 3],
                                              p.obs_pixel[2 * e:2 * e + 2])
        # pred = f d u: its FP32 rounding error scales with the focal length
        worst_r = max(worst_r, float(np.max(np.abs(r[2 * e:2 * e + 2] - r0)) / p.cameras[9 * c + 6]))
        worst_j = max(worst_j, float(np.max(np.abs(jc[18 * e:18 * e + 18] - jc0.ravel())) / np.max(np.abs(jc0))))
    assert worst_r < 1e-6 and worst_j < 2e-5, (worst_r, worst_j)


def test_batch_chol9_and_inverse3_match_exact_solves(gba, torch_cuda):
    """test_schur.cu gates: 64 random SPD blocks (A = M^T M + 9I / + 3I), max abs error <= 1e-9."""
    torch = torch_cuda
    rng = np.random.default_rng(42)
    N = 64
    A9 = np.empty((N, 9, 9))
    b9 = rng.uniform(-1, 1, (N, 9))
    for i in range(N):
        M = rng.uniform(-1, 1, (9, 9))
        A9[i] = M.T @ M + 9 * np.eye(9)
    x_ref = np.linalg.solve(A9, b9[..., None])[..., 0]
    dA, db = _dev(torch, A9), _dev(torch, b9)
    dx = torch.empty_like(db)
    ok = torch.empty(N, dtype=torch.int32, device="cuda")
    gba.batch_chol9_factor_solve(dA.data_ptr(), db.data_ptr(), dx.data_ptr(), ok.data_ptr(), N)
    torch.cuda.synchronize()
    assert ok.cpu().numpy().all()
    assert np.max(np.abs(dx.cpu().numpy() - x_ref)) <= 1e-9

    A3 = np.empty((N, 3, 3))
    for i in range(N):
        M = rng.uniform(-1, 1, (3, 3))
        A3[i] = M.T @ M + 3 * np.eye(3)
    dA3 = _dev(torch, A3)
    dinv = torch.empty_like(dA3)
    gba.batch_inverse3_spd(dA3.data_ptr(), dinv.data_ptr(), ok.data_ptr(), N)
    torch.cuda.synchronize()
    assert ok.cpu().numpy().all()
    assert np.max(np.abs(dinv.cpu().numpy() - np.linalg.inv(A3))) <= 1e-9

    # non-SPD input is reported, not silently solved
    bad = A9.copy()
    bad[5] = -np.eye(9)
    bad[9, 4, 4] = -1.0
    dA = _dev(torch, bad)
    gba.batch_chol9_factor_solve(dA.data_ptr(), db.data_ptr(), dx.data_ptr(), ok.data_ptr(), N)
    torch.cuda.synchronize()
    okv = ok.cpu().numpy()
    assert okv[5] == 0 and okv[9] == 0 and okv.sum() == N - 2


@pytest.mark.parametrize("n,lda", [(64, 64), (320, 320), (448, 512)])
def test_dense_potrf_potrs_match_numpy(gba, torch_cuda, n, lda):
    torch = torch_cuda
    rng = np.random.default_rng(n)
    M = rng.normal(size=(n, n))
    A = M @ M.T + n * np.eye(n)
    buf = np.zeros((n, lda))  # column j at buf[j, :n] -> column-major with leading dimension lda
    buf[:, :n] = A.T
    dA = _dev(torch, buf)
    info = torch.zeros(1, dtype=torch.int32, device="cuda")
    gba.dense_potrf(dA.data_ptr(), n, lda, info.data_ptr())
    torch.cuda.synchronize()
    assert int(info.item()) == 0
    L = np.tril(dA.cpu().numpy()[:, :n].T)
    assert rel_err(L, np.linalg.cholesky(A)) < 1e-12
    b = rng.normal(size=n)
    db = _dev(torch, b)
    gba.dense_potrs(dA.data_ptr(), n, lda, db.data_ptr(), info.data_ptr())
    torch.cuda.synchronize()
    assert rel_err(db.cpu().numpy(), np.linalg.solve(A, b)) < 1e-10


def test_dense_potrf_reports_failed_column(gba, torch_cuda):
    torch = torch_cuda
    n = 192
    A = np.eye(n) * 4.0
    A[130, 130] = -1.0
    dA = _dev(torch, A.T.copy())
    info = torch.zeros(1, dtype=torch.int32, device="cuda")
    gba.dense_potrf(dA.data_ptr(), n, n, info.data_ptr())
    torch.cuda.synchronize()
    assert int(info.item()) == 131


def _oracle_layout(gba, solver, prob):
    """Device buffers in the oracle's layout (observation order, full blocks)."""
    C, P, E = prob.num_cameras, prob.num_points, prob.num_observations
    Vp = solver.download("V").reshape(P, 6)
    V = np.empty((P, 3, 3))
    idx = [(0, 0, 0), (1, 1, 0), (2, 1, 1), (3, 2, 0), (4, 2, 1), (5, 2, 2)]
    for k, i, j in idx:
        V[:, i, j] = Vp[:, k]
        V[:, j, i] = Vp[:, k]
    order = solver.download("order")
    W = np.empty((E, 9, 3))
    W[order] = solver.download("W").reshape(E, 9, 3)
    return dict(U=solver.download("U").reshape(C, 9, 9), V=V, W=W, bc=solver.download("bc"),
                bp=solver.download("bp"))


def test_accumulate_plain_matches_oracle(gba, oracle, small):
    with gba.Solver(small, "plain") as s:
        sse = s.accumulate()
        dev = _oracle_layout(gba, s, small)
        sse2 = s.accumulate()
        U2 = s.download("U")
    ref = oracle.accumulate(small)
    assert abs(sse - ref["sse"]) <= 1e-12 * ref["sse"]
    for k in ("U", "V", "W", "bc", "bp"):
        assert rel_err(dev[k], ref[k]) < 1e-11, k
    # atomic-free reductions: bit-identical on a re-run
    assert sse2 == sse and np.array_equal(U2, dev["U"].ravel())


def test_schur_stages_match_oracle(gba, oracle, small):
    lam = 3e-3
    ref = oracle.schur_step(small, lam, threads=2, want_S=True)
    assert ref["status"] == 0
    C = small.num_cameras
    with gba.Solver(small, "plain") as s:
        s.accumulate()
        assert s.damp_invert_v(lam) == 0
        assert s.schur_dense(lam) == 0
        rhs = s.download("rhs")[:9 * C]
        dc = s.download("dc")
        denom = s.back_substitute(lam)
        dp = s.download("dp")
        tc = s.download("trial_cams")
    assert rel_err(rhs, ref["rhs"]) < 1e-10
    assert rel_err(dc, ref["dc"]) < 1e-9
    assert rel_err(dp, ref["dp"]) < 1e-9
    assert abs(denom - ref["denom"]) <= 1e-9 * abs(ref["denom"])
    np.testing.assert_allclose(tc, small.cameras + dc, rtol=0, atol=1e-12 * np.max(np.abs(tc)))


def test_assembled_S_matches_oracle(gba, oracle, small):
    """S before factorisation: check through its Cholesky factor (the device
    factors S in place) against the oracle's assembled S."""
    lam = 1e-2
    ref = oracle.schur_step(small, lam, threads=2, want_S=True)
    n = 9 * small.num_cameras
    S_ref = np.tril(ref["S"])
    S_ref = S_ref + np.tril(S_ref, -1).T
    with gba.Solver(small, "plain") as s:
        s.set_schur_layout("dense")
        _, _, _, n_pad = s.dims()
        s.accumulate()
        s.damp_invert_v(lam)
        assert s.schur_dense(lam) == 0
        Lfull = s.download("S").reshape(n_pad, n_pad).T  # column-major -> [row, col]
    L = np.tril(Lfull[:n, :n])
    assert rel_err(L @ L.T, S_ref) < 1e-10
    np.testing.assert_allclose(np.diag(Lfull)[n:], 1.0)


def test_nonspd_and_failed_factorisation_are_reported(gba, small):
    with gba.Solver(small, "plain") as s:
        s.accumulate()
        assert s.damp_invert_v(-1.5) == small.num_points  # every damped V block negative definite
        assert s.schur_dense(-1.5) > 0
        assert s.counters()[1] == small.num_points


def test_plain_lm_trajectory_matches_oracle_workload1(gba, oracle):
    """Workload 1 (16 / 22,000 / ~84k), 20 iterations: per-iteration cost 1e-9."""
    prob = gba.synthetic(1)
    ref, ref_cams, ref_pts = oracle.solve(prob, max_iterations=20)
    reader = gba.total_squared_error(prob) / 2
    run = prob.copy()
    res = gba.solve(run, max_iterations=20)
    assert abs(res.initial_cost - reader) <= 1e-9 * max(1.0, reader)
    assert res.anomalies == 0
    assert res.termination == ref["termination"]
    assert res.iterations == ref["iterations"]
    t_dev, t_ref = np.array(res.trajectory), np.array(ref["trajectory"])
    assert t_dev.shape == t_ref.shape
    assert np.max(np.abs(t_dev - t_ref) / t_ref) < 1e-9
    assert rel_err(run.cameras, ref_cams) < 1e-6


def test_launch_bounds_regression(gba):
    """tests/test_launch_bounds.cpp: P = 400,000 noise-free, every point must move."""
    prob = gba.launch_bounds_problem(400000)
    res = gba.solve(prob)
    assert res.initial_cost > 1.0
    assert res.termination == "CONVERGENCE"
    assert res.anomalies == 0
    assert res.final_cost < 1e-4 * res.initial_cost


def test_non_finite_observation_is_counted_and_skipped(gba, oracle):
    prob = gba.synthetic_custom(5, 400, 2, 5, 1.4, seed=8)
    prob.obs_pixel[10] = np.nan
    with gba.Solver(prob, "plain") as s:
        sse = s.accumulate()
        assert s.counters()[0] == 1
        U = s.download("U")
    ref = oracle.accumulate(prob)
    assert ref["anomalies"] == 1
    assert abs(sse - ref["sse"]) <= 1e-12 * ref["sse"]
    assert rel_err(U, ref["U"].ravel()) < 1e-11
    # every trial cost then sees the non-finite residual: all trials rejected
    res = gba.solve(prob.copy(), max_inner_trials=4)
    assert res.termination == "FAILURE"
    assert res.anomalies == 1 + 4
    assert res.trials == 4


def test_optimum_start_fails_after_all_trials(gba):
    """No step can lower a zero-noise optimum: all inner trials rejected -> FAILURE."""
    prob, truth = gba.synthetic(1, with_truth=True)
    zero = truth.copy()
    for e in range(zero.num_observations):
        c, q = zero.obs_camera[e], zero.obs_point[e]
        r = gba.snavely_residual(zero.cameras[9 * c:9 * c + 9], zero.points[3 * q:3 * q + 3], np.zeros(2))
        zero.obs_pixel[2 * e:2 * e + 2] = r
    res = gba.solve(zero)
    assert res.initial_cost < 1e-12
    assert res.termination in ("FAILURE", "CONVERGENCE")
    if res.termination == "FAILURE":
        assert res.trials == 16 and res.iterations == 0


def test_accumulate_huber_matches_oracle(gba, oracle, small):
    """Huber loss (first-order corrector): rows scaled by sqrt(rho'), SSE = sum of rho."""
    d = 2.0
    with gba.Solver(small, "plain") as s:
        s.set_loss("huber", d)
        sse = s.accumulate()
        dev = _oracle_layout(gba, s, small)
    assert abs(sse - oracle.cost(small, huber_delta=d)) <= 1e-12 * sse
    ref = oracle.accumulate(small, huber_delta=d)
    assert abs(sse - ref["sse"]) <= 1e-12 * ref["sse"]
    for k in ("U", "V", "W", "bc", "bp"):
        assert rel_err(dev[k], ref[k]) < 1e-11, k


def test_plain_huber_lm_trajectory_matches_oracle_workload1(gba, oracle):
    """Workload 1 under the Huber loss (delta 1 px), 15 iterations: per-iteration cost 1e-9."""
    prob = gba.synthetic(1)
    ref, ref_cams, _ = oracle.solve(prob, max_iterations=15, huber_delta=1.0)
    run = prob.copy()
    res = gba.solve(run, max_iterations=15, loss="huber", huber_delta=1.0)
    assert abs(res.initial_cost - oracle.cost(prob, huber_delta=1.0) / 2) <= 1e-9 * res.initial_cost
    assert res.anomalies == 0
    assert res.termination == ref["termination"]
    assert res.iterations == ref["iterations"]
    t_dev, t_ref = np.array(res.trajectory), np.array(ref["trajectory"])
    assert t_dev.shape == t_ref.shape
    assert np.max(np.abs(t_dev - t_ref) / t_ref) < 1e-9
    assert rel_err(run.cameras, ref_cams) < 1e-6


@pytest.mark.parametrize("form", ["plain", "mixed"])
def test_solver_create_rejects_bad_indices(gba, form):
    """Observation indices are range-checked on the device before any kernel
    indexes with them; a bad one is an invalid-argument status (1)."""
    prob = gba.synthetic_custom(3, 10, 2, 3, 1.5, seed=1)
    for field, value in (("obs_point", 10), ("obs_point", -1), ("obs_camera", 3)):
        bad = prob.copy()
        getattr(bad, field)[0] = value
        with pytest.raises(gba.GbaError) as ei:
            gba.Solver(bad, form)
        assert ei.value.status == 1
        with pytest.raises(gba.GbaError) as ei:
            gba.solve(bad, form=form)
        assert ei.value.status == 1
    gba.Solver(prob, form).close()  # the device is still usable


def test_long_tracks_plain_schur_step_matches_oracle(gba, oracle):
    """Points observed ~300 times (point chunks longer than one CTA pass,
    ~45,000 edge pairs per point in the S assembly): FP64 step vs the oracle."""
    prob = gba.synthetic_custom(320, 40, 290, 310, 1.2, seed=3)
    lam = 1e-3
    ref = oracle.schur_step(prob, lam, threads=4)
    assert ref["status"] == 0
    with gba.Solver(prob, "plain") as s:
        s.accumulate()
        assert s.damp_invert_v(lam) == 0
        assert s.schur_dense(lam) == 0
        dc = s.download("dc")
        denom = s.back_substitute(lam)
        dp = s.download("dp")
    assert rel_err(dc, ref["dc"]) < 1e-9
    assert rel_err(dp, ref["dp"]) < 1e-9
    assert abs(denom - ref["denom"]) <= 1e-9 * abs(ref["denom"])
