"""GPU: the learned coarse-basis MLP kernels against the CPU oracle
(oracle/mlp_oracle.py), the two-level PCG that uses the basis, and training on
systems the plain solver assembles.

Tolerances: the GPU GEMMs take BF16 operands and accumulate in FP32; the oracle
rounds the same operands to BF16 and sums exactly, so forward outputs agree to
1e-4 and gradients to 2e-3 (relative, max-norm). The two-level preconditioner
changes how PCG converges, not what it converges to: refined to 1e-10, its
step equals block-Jacobi's to 1e-7.
"""
import numpy as np
import pytest

from conftest import PKG

pytestmark = pytest.mark.gpu

MODEL = PKG / "models" / "coarse_mlp.bin"


@pytest.fixture(scope="module")
def mlp_oracle():
    import mlp_oracle

    return mlp_oracle


def _rel(a, b):
    return float(np.max(np.abs(np.asarray(a, np.float64) - b)) / max(np.max(np.abs(b)), 1e-30))


@pytest.fixture(scope="module")
def system(gba, torch_cuda):
    """Features, cameras, diagonal-block factors and the lowest eigenvectors of
    the Jacobi-preconditioned S from one plain-form trial of a small problem."""
    import train_preconditioner as tp

    torch = torch_cuda
    C = 40
    prob = gba.synthetic_custom(C, 3000, 2, 8, 1.6, seed=17)
    lam = 1e-3
    with gba.Solver(prob, "plain") as s:
        s.set_schur_layout("dense")
        gba.solver_set_harvest(s, True)
        s.accumulate()
        assert s.damp_invert_v(lam) == 0
        assert s.schur_dense(lam) == 0
        _, _, _, n_pad = s.dims()
        feat = torch.empty((C, 64), dtype=torch.float32, device="cuda")
        gba.solver_features(s, lam, feat.data_ptr())
        torch.cuda.synchronize()
        Sdiag = s.download("Sdiag").reshape(C, 9, 9)
        L = np.tril(s.download("S").reshape(n_pad, n_pad).T[:9 * C, :9 * C])
        cams, _ = s.get_params()
    ev, V, Bl = tp.jacobi_eigvecs(L, Sdiag, C, tp.M_EIG)
    return dict(feat=feat, f=feat.cpu().numpy(), cams=cams.reshape(C, 9), B=Bl, V=V, ev=ev, C=C)


def test_features_layout(system):
    f, cams = system["f"], system["cams"]
    assert np.isfinite(f).all()
    assert np.all(np.abs(f[:, :36]) <= 1.0 + 1e-5)  # correlations of an SPD block
    assert np.all((f[:, 36:45] > 0) & (f[:, 36:45] <= 1.0 + 1e-6))  # diagonal share after elimination
    np.testing.assert_allclose(f[:, 49:52], 3 * cams[:, :3], rtol=1e-6, atol=1e-7)
    np.testing.assert_allclose(f[:, 52:55], 0.5 * cams[:, 3:6], rtol=1e-6, atol=1e-7)
    np.testing.assert_allclose(f[:, 55], (cams[:, 6] - 500) / 100, rtol=1e-5, atol=1e-6)
    assert np.all(f[:, 58:] == 0)


def _random_params(mlp_oracle, seed):
    rng = np.random.default_rng(seed)
    p = mlp_oracle.unpack(np.zeros(mlp_oracle.N_PARAMS))
    p["W1"][:, :mlp_oracle.USED_IN] = rng.normal(0, 0.2, (128, mlp_oracle.USED_IN))
    p["b1"][:] = rng.normal(0, 0.1, 128)
    p["W2"][:] = rng.normal(0, 0.12, (128, 128))
    p["b2"][:] = rng.normal(0, 0.1, 128)
    p["W3"][:81] = rng.normal(0, 0.05, (81, 128))
    p["b3"][:81] = rng.normal(0, 0.05, 81)
    return mlp_oracle.pack(p).astype(np.float32)


def test_forward_matches_oracle(gba, torch_cuda, mlp_oracle, system):
    torch = torch_cuda
    C = system["C"]
    m = gba.Mlp(capacity=64)
    params = _random_params(mlp_oracle, 1)
    m.set_params(params)
    out = torch.empty((C, 96), dtype=torch.float32, device="cuda")
    m.forward(system["feat"].data_ptr(), C, out.data_ptr())
    ref, _ = mlp_oracle.forward(params.astype(np.float64), system["f"].astype(np.float64))
    assert _rel(out.cpu().numpy(), ref) < 1e-4


def test_backward_matches_oracle(gba, torch_cuda, mlp_oracle, system):
    """Parameter gradients from the closed-form loss gradient of a real system."""
    import train_preconditioner as tp

    torch = torch_cuda
    C = system["C"]
    m = gba.Mlp(capacity=64)
    params = _random_params(mlp_oracle, 2)
    m.set_params(params)
    out = torch.empty((C, 96), dtype=torch.float32, device="cuda")
    m.forward(system["feat"].data_ptr(), C, out.data_ptr())
    O = out.cpu().numpy()
    _, dO, _ = tp.coarse_loss_and_grad(O, system["cams"], system["B"], system["V"])
    d = torch.from_numpy(dO.astype(np.float32)).cuda()
    m.backward(system["feat"].data_ptr(), d.data_ptr(), C)
    g_dev = m.grads()
    ref = mlp_oracle.backward(params.astype(np.float64), system["f"].astype(np.float64), dO.astype(np.float32))
    dev_p, ref_p = mlp_oracle.unpack(g_dev.astype(np.float64)), mlp_oracle.unpack(ref)
    for name in ("W1", "b1", "W2", "b2", "W3", "b3"):
        assert _rel(dev_p[name], ref_p[name]) < 2e-3, name


def test_adam_step_matches_reference_update(gba, torch_cuda, mlp_oracle, system):
    torch = torch_cuda
    C = system["C"]
    m = gba.Mlp(capacity=64)
    p0 = _random_params(mlp_oracle, 4)
    m.set_params(p0)
    out = torch.empty((C, 96), dtype=torch.float32, device="cuda")
    m.forward(system["feat"].data_ptr(), C, out.data_ptr())
    dO = torch.randn((C, 96), dtype=torch.float32, device="cuda", generator=torch.Generator("cuda").manual_seed(1))
    m.backward(system["feat"].data_ptr(), dO.data_ptr(), C)
    g = m.grads().astype(np.float64)
    m.adam_step(1e-2, 0.9, 0.999, 1e-8)
    mh = 0.1 * g / (1 - 0.9)
    vh = 0.001 * g * g / (1 - 0.999)
    expect = p0 - 1e-2 * mh / (np.sqrt(vh) + 1e-8)
    assert _rel(m.params(), expect) < 1e-5


def test_training_on_gpu_reduces_coarse_loss(gba, torch_cuda, system):
    """The library's forward / backward / Adam kernels with the closed-form loss
    gradient: the eigenvector share outside the basis drops."""
    import train_preconditioner as tp

    torch = torch_cuda
    C = system["C"]
    m = gba.Mlp(seed=5, capacity=64)
    out = torch.empty((C, 96), dtype=torch.float32, device="cuda")
    losses = []
    for step in range(400):
        m.forward(system["feat"].data_ptr(), C, out.data_ptr())
        loss, dO, _ = tp.coarse_loss_and_grad(out.cpu().numpy(), system["cams"], system["B"], system["V"])
        losses.append(loss)
        d = torch.from_numpy(dO.astype(np.float32)).cuda()
        m.backward(system["feat"].data_ptr(), d.data_ptr(), C)
        m.adam_step(2e-3)
    assert losses[-1] < 0.5 * losses[0], (losses[0], losses[-1])


@pytest.fixture(scope="module")
def random_model(gba, tmp_path_factory):
    path = tmp_path_factory.mktemp("mlp") / "random.bin"
    m = gba.Mlp(seed=11, capacity=16)
    m.save(path)
    return path


@pytest.mark.parametrize("tracks", ["short", "long"])
def test_two_level_pcg_refined_step_equals_block_jacobi(gba, random_model, tracks):
    """Any full-rank basis gives an SPD preconditioner: forced on, the refined
    Schur step equals the block-Jacobi one (same system, refined to 1e-10).
    Long tracks (40 to 300 observations) take the coarse product's list and
    single-point passes besides the warp pass."""
    prob = (gba.synthetic_custom(30, 4000, 2, 8, 1.6, seed=23) if tracks == "short"
            else gba.synthetic_custom(400, 1500, 40, 300, 1.0, seed=23))
    lam = 1e-3
    steps = []
    for mode in ("block-jacobi", "learned"):
        with gba.Solver(prob, "learned") as s:
            s.load_model(random_model)
            s.set_preconditioner(mode)
            s.accumulate()
            assert s.damp_invert_v(lam) == 0
            iters, nsteps, relres = s.schur_pcg(lam, learned=True, refine_tol=1e-10, pcg_tol=1e-4,
                                                pcg_max_iters=500)
            assert relres <= 1e-10, (mode, relres)
            steps.append(s.download("dc"))
    assert _rel(steps[1], steps[0]) < 1e-7


def test_two_level_lm_solve_matches_oracle_cost(gba, oracle, random_model):
    """A whole learned-form solve with the coarse correction forced on (an
    untrained basis): initial cost = reader cost, final cost within 0.1% of the
    FP64 oracle's."""
    prob = gba.synthetic(1)
    ref, _, _ = oracle.solve(prob, max_iterations=20)
    with gba.Solver(prob, "learned") as s:
        s.load_model(random_model)
        s.set_preconditioner("learned")
        r = s.run(max_iterations=20, form="learned", model_path=str(random_model))
    assert abs(r.initial_cost - ref["initial_cost"]) <= 1e-9 * ref["initial_cost"]
    assert r.anomalies == 0
    assert r.final_cost <= ref["final_cost"] * (1 + 1e-3)


@pytest.mark.skipif(not MODEL.exists(), reason="trained model not present")
def test_learned_lm_reaches_oracle_cost_workload1(gba, oracle):
    prob = gba.synthetic(1)
    ref, _, _ = oracle.solve(prob, max_iterations=20)
    learned = gba.solve(prob.copy(), max_iterations=20, form="learned", model_path=str(MODEL))
    assert learned.anomalies == 0
    assert learned.final_cost <= ref["final_cost"] * (1 + 1e-3)
    assert learned.learned_choice in (1, 2)


@pytest.mark.skipif(not MODEL.exists(), reason="trained model not present")
def test_learned_huber_reaches_oracle_cost_workload1(gba, oracle):
    """Huber loss through the learned form (judged preconditioner on the robust
    system): final robust cost within 0.1% of the oracle's."""
    prob = gba.synthetic(1)
    ref, _, _ = oracle.solve(prob, max_iterations=15, huber_delta=1.0)
    res = gba.solve(prob.copy(), max_iterations=15, form="learned", model_path=str(MODEL), loss="huber",
                    huber_delta=1.0)
    assert abs(res.initial_cost - ref["initial_cost"]) <= 1e-9 * ref["initial_cost"]
    assert res.anomalies == 0
    assert res.final_cost <= ref["final_cost"] * (1 + 1e-3)
    assert res.learned_choice in (1, 2)
