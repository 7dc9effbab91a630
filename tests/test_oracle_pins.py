"""CPU: pins the oracle (CPU restatement of the reference LM) to the reference's
own code and golden cases, and the host side of the library to the oracle.

Reference tests followed: tests/test_vs_ceres.cpp:31-74 (finite-difference
Jacobian on two golden cases), tests/test_schur.cu (SPD factor / inverse to
1e-9), the initial-cost identity of benchmarks/bench_bal.cpp:87-94.
"""
import json

import numpy as np
import pytest

from conftest import GOLDEN, rel_err


def _fd_jacobian(fn, cam, pt, obs, eps=1e-6):
    """Central differences of fn(cam, pt, obs) -> r2 (reference test_vs_ceres.cpp:50-69)."""
    cam, pt = np.array(cam, float), np.array(pt, float)
    Jc, Jp = np.zeros((2, 9)), np.zeros((2, 3))
    for j in range(9):
        a, b = cam.copy(), cam.copy()
        a[j] += eps
        b[j] -= eps
        Jc[:, j] = (fn(a, pt, obs) - fn(b, pt, obs)) / (2 * eps)
    for j in range(3):
        a, b = pt.copy(), pt.copy()
        a[j] += eps
        b[j] -= eps
        Jp[:, j] = (fn(cam, a, obs) - fn(cam, b, obs)) / (2 * eps)
    return Jc, Jp


def _fd_err(J, Jfd):
    return float(np.max(np.abs(J - Jfd) / np.maximum(1.0, np.abs(J))))


def test_oracle_residual_matches_reference_golden(oracle):
    g = json.loads((GOLDEN / "residual_golden.json").read_text())
    worst = 0.0
    for e in g["edges"]:
        r = oracle.residual(e["cam"], e["pt"], e["obs"])
        ref = np.array(e["residual"])
        worst = max(worst, float(np.max(np.abs(r - ref)) / max(1.0, np.max(np.abs(ref)))))
    # Same model; the CPU reader drops the first-order a x X term below |a| = 1e-12
    # and uses theta > 1e-12 instead of theta^2 > 1e-24: ~1e-12 px at most.
    assert worst < 1e-9, worst


def test_oracle_residual_matches_reference_compiled(oracle):
    try:
        ref = oracle.ReferenceReader()
    except FileNotFoundError:
        pytest.skip("reference reader not built here (reference checkout absent)")
    rng = np.random.default_rng(5)
    for _ in range(100):
        cam = np.concatenate([rng.normal(0, 0.5, 3), rng.normal(0, 1, 3), [500.0], rng.normal(0, 0.05, 2)])
        pt = rng.normal(0, 3, 3) - np.array([0, 0, 8.0])
        obs = rng.normal(0, 100, 2)
        np.testing.assert_allclose(oracle.residual(cam, pt, obs), ref.snavely_residual(cam, pt, obs), rtol=1e-13,
                                   atol=1e-9)


@pytest.mark.parametrize("which", [0, 1])
def test_oracle_jacobian_vs_finite_differences(oracle, which):
    case = json.loads((GOLDEN / "fd_cases.json").read_text())["cases"][which]
    cam, pt, obs = case[:9], case[9:12], case[12:14]
    _, Jc, Jp = oracle.residual_jacobian(cam, pt, obs)
    Jc_fd, Jp_fd = _fd_jacobian(oracle.residual, cam, pt, obs)
    assert max(_fd_err(Jc, Jc_fd), _fd_err(Jp, Jp_fd)) < 1e-5


@pytest.mark.parametrize("which", [0, 1])
def test_library_host_jacobian_vs_finite_differences(gba, which):
    """gba_edge_residual_jacobian_host: the reference FD gate (rel err < 1e-5)."""
    case = json.loads((GOLDEN / "fd_cases.json").read_text())["cases"][which]
    cam, pt, obs = case[:9], case[9:12], case[12:14]
    _, Jc, Jp = gba.edge_residual_jacobian_host(cam, pt, obs)
    fn = lambda c, p, o: gba.edge_residual_jacobian_host(c, p, o)[0]  # noqa: E731
    Jc_fd, Jp_fd = _fd_jacobian(fn, cam, pt, obs)
    assert max(_fd_err(Jc, Jc_fd), _fd_err(Jp, Jp_fd)) < 1e-5


def test_library_jacobian_matches_oracle_derivation(gba, oracle):
    """The library's left-Jacobian derivation equals the reference's w-derivative one."""
    rng = np.random.default_rng(7)
    worst = 0.0
    for i in range(500):
        cam = np.concatenate([rng.normal(0, 0.4, 3), rng.normal(0, 1, 3), [rng.uniform(300, 700)],
                              rng.normal(0, 0.05, 1), rng.normal(0, 0.005, 1)])
        if i % 50 == 0:
            cam[:3] = rng.normal(0, 1e-14, 3)  # first-order branch
        pt = np.array([rng.uniform(-3, 3), rng.uniform(-3, 3), rng.uniform(-12, -3)])
        obs = rng.normal(0, 300, 2)
        r1, jc1, jp1 = gba.edge_residual_jacobian_host(cam, pt, obs)
        r2, jc2, jp2 = oracle.residual_jacobian(cam, pt, obs)
        for a, b in ((r1, r2), (jc1, jc2), (jp1, jp2)):
            worst = max(worst, float(np.max(np.abs(a - b)) / max(1.0, np.max(np.abs(b)))))
    assert worst < 1e-9, worst


def test_library_reader_and_sse_match_reference_golden(gba):
    meta = json.loads((GOLDEN / "tiny_problem.json").read_text())
    prob = gba.load_bal(GOLDEN / "tiny_problem.txt")
    assert (prob.num_cameras, prob.num_points, prob.num_observations) == (
        meta["num_cameras"], meta["num_points"], meta["num_observations"])
    sse = gba.total_squared_error(prob)
    assert abs(sse - meta["total_squared_error"]) <= 1e-12 * abs(meta["total_squared_error"])


def test_library_reader_matches_reference_reader(gba, oracle, tmp_path):
    try:
        ref = oracle.ReferenceReader()
    except FileNotFoundError:
        pytest.skip("reference reader not built here")
    cams, pts, oc, op, px = ref.load_bal(GOLDEN / "tiny_problem.txt")
    prob = gba.load_bal(GOLDEN / "tiny_problem.txt")
    for a, b in zip(prob.arrays(), (cams, pts, oc, op, px)):
        np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("text,ok", [
    ("1 1 1\n0 0 1.5 2.5\n" + "1\n" * 9 + "1\n2\n3\n", True),
    ("0 1 1\n0 0 1 1\n", False),                       # bad header
    ("1 1 1\n0 1 1.5 2.5\n" + "1\n" * 12, False),      # point index out of range
    ("1 1 1\n0 0 1.5 2.5\n" + "1\n" * 12 + "7\n", False),  # trailing garbage
    ("1 1 1\n0 0 1.5 x\n" + "1\n" * 12, False),        # malformed number
    ("1 1 1\n0 0 1.5 2.5\n" + "1\n" * 11, False),      # truncated
])
def test_reader_validation(gba, tmp_path, text, ok):
    """Reader error behaviour of the reference (src/bal_reader.cpp:66-98)."""
    f = tmp_path / "p.txt"
    f.write_text(text)
    if ok:
        prob = gba.load_bal(f)
        assert prob.num_observations == 1 and prob.obs_pixel.tolist() == [1.5, 2.5]
    else:
        with pytest.raises(gba.GbaError):
            gba.load_bal(f)


def test_oracle_cholesky_matches_numpy(oracle):
    rng = np.random.default_rng(3)
    n = 150
    M = rng.normal(size=(n, n))
    A = M @ M.T + n * np.eye(n)
    colmajor = np.asfortranarray(A).ravel(order="F").copy()
    assert oracle.cholesky(colmajor, n, 2) == 0
    L = np.tril(colmajor.reshape(n, n, order="F"))
    assert rel_err(L, np.linalg.cholesky(A)) < 1e-12
    bad = -np.eye(n).ravel()
    assert oracle.cholesky(bad, n, 1) == 1


def test_oracle_schur_step_matches_dense_normal_equations(gba, oracle):
    """The oracle's Schur step equals the full damped Gauss-Newton solve (numpy)."""
    prob = gba.synthetic_custom(4, 60, 2, 4, 1.5, seed=3)
    lam = 1e-2
    ne = oracle.accumulate(prob)
    C, P = prob.num_cameras, prob.num_points
    n = 9 * C + 3 * P
    H = np.zeros((n, n))
    b = np.concatenate([ne["bc"], ne["bp"]])
    for c in range(C):
        H[9 * c:9 * c + 9, 9 * c:9 * c + 9] = ne["U"][c]
    for p in range(P):
        H[9 * C + 3 * p:9 * C + 3 * p + 3, 9 * C + 3 * p:9 * C + 3 * p + 3] = ne["V"][p]
    for e in range(prob.num_observations):
        c, p = prob.obs_camera[e], prob.obs_point[e]
        H[9 * c:9 * c + 9, 9 * C + 3 * p:9 * C + 3 * p + 3] += ne["W"][e]
        H[9 * C + 3 * p:9 * C + 3 * p + 3, 9 * c:9 * c + 9] += ne["W"][e].T
    d = np.diag(H).copy()
    H[np.diag_indices(n)] += lam * np.where(d > 0, d, 1e-12)
    x = np.linalg.solve(H, b)
    st = oracle.schur_step(prob, lam, threads=2)
    assert st["status"] == 0
    assert rel_err(st["dc"], x[:9 * C]) < 1e-8
    assert rel_err(st["dp"], x[9 * C:]) < 1e-8


def test_back_substitution_residual_identity(gba, oracle):
    """The identity behind the mixed forms' last refinement check: for any dc,
    with dp = V'^-1 (bp - W^T dc), the Schur residual rhs - S dc equals
    bc - U_lambda dc - W dp (numpy FP64 on the oracle's normal equations)."""
    prob = gba.synthetic_custom(5, 200, 2, 5, 1.5, seed=11)
    lam = 1e-3
    ne = oracle.accumulate(prob)
    C, P = prob.num_cameras, prob.num_points
    U = ne["U"].copy()
    V = ne["V"].copy()
    for c in range(C):
        d = np.diag(U[c]).copy()
        U[c][np.diag_indices(9)] += lam * np.where(d > 0, d, 1e-12)
    for q in range(P):
        d = np.diag(V[q]).copy()
        V[q][np.diag_indices(3)] += lam * np.where(d > 0, d, 1e-12)
    Vinv = np.linalg.inv(V)
    W = np.zeros((9 * C, 3 * P))
    for e in range(prob.num_observations):
        c, q = prob.obs_camera[e], prob.obs_point[e]
        W[9 * c:9 * c + 9, 3 * q:3 * q + 3] += ne["W"][e]
    Ub = np.zeros((9 * C, 9 * C))
    Vb = np.zeros((3 * P, 3 * P))
    for c in range(C):
        Ub[9 * c:9 * c + 9, 9 * c:9 * c + 9] = U[c]
    for q in range(P):
        Vb[3 * q:3 * q + 3, 3 * q:3 * q + 3] = Vinv[q]
    S = Ub - W @ Vb @ W.T
    rhs = ne["bc"] - W @ Vb @ ne["bp"]
    dc = np.random.default_rng(2).standard_normal(9 * C) * 1e-3
    dp = Vb @ (ne["bp"] - W.T @ dc)
    lhs = rhs - S @ dc
    rhs_form = ne["bc"] - Ub @ dc - W @ dp
    assert np.linalg.norm(lhs - rhs_form) <= 1e-12 * max(np.linalg.norm(ne["bc"]), np.linalg.norm(Ub @ dc))


def test_oracle_lm_converges_on_small_problem(gba, oracle):
    prob = gba.synthetic_custom(6, 400, 2, 6, 1.5, seed=4)
    res, _, _ = oracle.solve(prob, max_iterations=30, threads=2)
    assert res["anomalies"] == 0
    assert res["termination"] in ("CONVERGENCE", "MAX_ITERATIONS")
    traj = res["trajectory"]
    assert all(b < a for a, b in zip(traj, traj[1:]))
    # noise is N(0,1) px: the optimum is near E px^2 / 2 per observation
    assert res["final_cost"] < 0.75 * prob.num_observations
    assert abs(res["initial_cost"] - gba.total_squared_error(prob) / 2) <= 1e-9 * res["initial_cost"]


def test_mlp_oracle_backward_through_coarse_loss_vs_finite_differences():
    """The oracle's backward pass, fed the closed-form gradient of the coarse
    loss (train_preconditioner.coarse_loss_and_grad), against central
    differences of the composed loss w.r.t. the network parameters (FP64)."""
    import mlp_oracle
    import train_preconditioner as tp

    rng = np.random.default_rng(12)
    C, m = 5, 4
    V, _ = np.linalg.qr(rng.standard_normal((9 * C, m)))
    Bl = np.tril(rng.standard_normal((C, 9, 9))) + 3 * np.eye(9)[None]
    cams = np.zeros((C, 9))
    cams[:, 6] = rng.uniform(400, 600, C)
    feat = np.zeros((C, 64))
    feat[:, :mlp_oracle.USED_IN] = rng.normal(0, 0.5, (C, mlp_oracle.USED_IN))
    p = mlp_oracle.unpack(np.zeros(mlp_oracle.N_PARAMS))
    p["W1"][:, :mlp_oracle.USED_IN] = rng.normal(0, 0.3, (128, mlp_oracle.USED_IN))
    p["b1"][:] = 0.05
    p["W2"][:] = rng.normal(0, 0.1, (128, 128))
    p["W3"][:81] = rng.normal(0, 0.05, (81, 128))
    p["b3"][:81] = rng.normal(0, 0.05, 81)
    flat = mlp_oracle.pack(p)

    def loss_at(v):
        o, _ = mlp_oracle.forward(v, feat, emulate_bf16=False)
        return tp.coarse_loss_and_grad(o, cams, Bl, V)[0]

    o, _ = mlp_oracle.forward(flat, feat, emulate_bf16=False)
    _, dO, _ = tp.coarse_loss_and_grad(o, cams, Bl, V)
    grad = mlp_oracle.backward(flat, feat, dO, emulate_bf16=False)
    sizes = np.cumsum([0] + [int(np.prod(s)) for _, s in mlp_oracle.SIZES])
    idx = [sizes[0] + 5, sizes[1] + 3, sizes[2] + 700, sizes[3] + 9, sizes[4] + 129, sizes[5] + 2]
    for i in idx:
        e = np.zeros_like(flat)
        e[i] = 1e-5
        fd = (loss_at(flat + e) - loss_at(flat - e)) / 2e-5
        # the forward stores activations in FP32, so differences resolve ~1e-7
        assert abs(fd - grad[i]) < 1e-4 * max(1.0, abs(fd)) + 1e-6, (i, fd, grad[i])


def test_oracle_huber_cost_matches_per_observation_rho(gba, oracle):
    """Huber cost = sum rho(|r|^2), rho(s) = s for s <= d^2 else 2 d sqrt(s) - d^2; a huge d is the plain cost."""
    prob = gba.synthetic_custom(4, 60, 2, 4, 1.5, seed=3)
    d = 2.0
    s = np.array([np.sum(oracle.residual(prob.cameras[9 * c:9 * c + 9], prob.points[3 * p:3 * p + 3],
                                         prob.obs_pixel[2 * e:2 * e + 2]) ** 2)
                  for e, (c, p) in enumerate(zip(prob.obs_camera, prob.obs_point))])
    rho = np.where(s <= d * d, s, 2 * d * np.sqrt(s) - d * d)
    assert abs(oracle.cost(prob, huber_delta=d) - rho.sum()) <= 1e-12 * rho.sum()
    assert oracle.cost(prob, huber_delta=1e12) == oracle.cost(prob)
    assert oracle.cost(prob, huber_delta=d) < oracle.cost(prob)


@pytest.mark.parametrize("k", [0, 2, 4, 7, 8])
def test_oracle_huber_gradient_vs_finite_differences(gba, oracle, k):
    """With the first-order corrector, b = -grad(cost / 2) exactly (cameras; points likewise)."""
    prob = gba.synthetic_custom(4, 60, 2, 4, 1.5, seed=3)
    d = 2.0
    ne = oracle.accumulate(prob, huber_delta=d)
    for cam in range(prob.num_cameras):
        i = 9 * cam + k
        h = 1e-6 * max(1.0, abs(prob.cameras[i]))
        cp, cm = prob.cameras.copy(), prob.cameras.copy()
        cp[i] += h
        cm[i] -= h
        fd = 0.5 * (oracle.cost(prob, cp, None, d) - oracle.cost(prob, cm, None, d)) / (2 * h)
        assert abs(fd + ne["bc"][i]) <= 1e-5 * max(1.0, abs(fd)), (cam, k, fd, ne["bc"][i])
    for p in range(0, prob.num_points, 7):
        i = 3 * p + k % 3
        h = 1e-6 * max(1.0, abs(prob.points[i]))
        pp, pm = prob.points.copy(), prob.points.copy()
        pp[i] += h
        pm[i] -= h
        fd = 0.5 * (oracle.cost(prob, None, pp, d) - oracle.cost(prob, None, pm, d)) / (2 * h)
        assert abs(fd + ne["bp"][i]) <= 1e-5 * max(1.0, abs(fd)), (p, fd, ne["bp"][i])


def test_oracle_huber_lm_decreases_robust_cost(gba, oracle):
    prob = gba.synthetic_custom(6, 400, 2, 6, 1.5, seed=4)
    res, _, _ = oracle.solve(prob, max_iterations=20, threads=2, huber_delta=1.0)
    assert res["anomalies"] == 0
    traj = res["trajectory"]
    assert all(b < a for a, b in zip(traj, traj[1:]))
    assert abs(res["initial_cost"] - oracle.cost(prob, huber_delta=1.0) / 2) <= 1e-12 * res["initial_cost"]
