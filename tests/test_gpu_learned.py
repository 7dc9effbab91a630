"""GPU: the learned block-Jacobi MLP kernels against the CPU oracle
(oracle/mlp_oracle.py), and the trained network against the method without it.

Tolerances: the GPU GEMMs take BF16 operands and accumulate in FP32; the oracle
rounds the same operands to BF16 and sums exactly, so forward outputs agree to
1e-4 and gradients to 2e-3 (relative, max-norm), the loss to 1e-5.
"""
import json
from pathlib import Path

import numpy as np
import pytest

from conftest import PKG

pytestmark = pytest.mark.gpu

MODEL = PKG / "models" / "bj_mlp.bin"


@pytest.fixture(scope="module")
def mlp_oracle():
    import mlp_oracle

    return mlp_oracle


def _rel(a, b):
    return float(np.max(np.abs(np.asarray(a, np.float64) - b)) / max(np.max(np.abs(b)), 1e-30))


@pytest.fixture(scope="module")
def batch(gba, torch_cuda, mlp_oracle):
    """Real (S_cc, g, x*) triples from one plain-form trial of a small problem."""
    torch = torch_cuda
    prob = gba.synthetic_custom(40, 3000, 2, 8, 1.6, seed=17)
    lam = 1e-3
    with gba.Solver(prob, "plain") as s:
        gba.solver_set_harvest(s, True)
        s.accumulate()
        assert s.damp_invert_v(lam) == 0
        assert s.schur_dense(lam) == 0
        feat = torch.empty((40, 64), dtype=torch.float32, device="cuda")
        gba.solver_features(s, lam, feat.data_ptr())
        torch.cuda.synchronize()
        Sdiag = s.download("Sdiag").reshape(40, 9, 9)
        g = s.download("rhs")[:360].reshape(40, 9)
        x = s.download("dc").reshape(40, 9)
    S, L, gh, xh = [], [], [], []
    for c in range(40):
        a, b, gg, xx = mlp_oracle.scaled_sample(Sdiag[c], g[c], x[c])
        S.append(a)
        L.append(b)
        gh.append(gg)
        xh.append(xx)
    host = dict(f=feat.cpu().numpy(), S=np.array(S), L=np.array(L), g=np.array(gh), x=np.array(xh))
    dev = {k: torch.from_numpy(np.ascontiguousarray(v)).cuda() for k, v in host.items()}
    return host, dev


def test_features_are_finite_and_scaled(batch):
    host, _ = batch
    f = host["f"]
    assert np.isfinite(f).all()
    assert np.all(np.abs(f[:, :36]) <= 1.0 + 1e-5)  # correlations of an SPD block
    assert np.all((f[:, 36:45] > 0) & (f[:, 36:45] <= 1.0 + 1e-6))  # diagonal share after elimination
    assert np.all(f[:, 49:] == 0)


def _random_params(gba, mlp_oracle, seed):
    rng = np.random.default_rng(seed)
    p = mlp_oracle.unpack(np.zeros(mlp_oracle.N_PARAMS))
    p["W1"][:, :49] = rng.normal(0, 0.2, (128, 49))
    p["b1"][:] = rng.normal(0, 0.1, 128)
    p["W2"][:] = rng.normal(0, 0.12, (128, 128))
    p["b2"][:] = rng.normal(0, 0.1, 128)
    p["W3"][:45] = rng.normal(0, 0.05, (45, 128))
    p["b3"][:45] = rng.normal(0, 0.05, 45)
    return mlp_oracle.pack(p).astype(np.float32)


def test_forward_matches_oracle(gba, torch_cuda, mlp_oracle, batch):
    torch = torch_cuda
    host, dev = batch
    m = gba.Mlp(capacity=64)
    params = _random_params(gba, mlp_oracle, 1)
    m.set_params(params)
    out = torch.empty((40, 48), dtype=torch.float32, device="cuda")
    m.forward(dev["f"].data_ptr(), 40, out.data_ptr())
    ref, _ = mlp_oracle.forward(params.astype(np.float64), host["f"].astype(np.float64))
    assert _rel(out.cpu().numpy(), ref) < 1e-4


def test_loss_and_gradients_match_oracle(gba, torch_cuda, mlp_oracle, batch):
    host, dev = batch
    m = gba.Mlp(capacity=64)
    params = _random_params(gba, mlp_oracle, 2)
    m.set_params(params)
    loss, base = m.loss_grad(*(dev[k].data_ptr() for k in ("f", "S", "L", "g", "x")), 40)
    g_dev = m.grads()
    ref_loss, ref_base, ref_g = mlp_oracle.loss_and_grads(params.astype(np.float64), host["f"].astype(np.float64),
                                                           host["S"], host["L"], host["g"], host["x"])
    assert abs(loss - ref_loss) <= 1e-5 * max(ref_loss, 1e-12)
    assert abs(base - ref_base) <= 1e-9 * max(ref_base, 1e-12)
    ref_p = mlp_oracle.unpack(ref_g)
    dev_p = mlp_oracle.unpack(g_dev.astype(np.float64))
    for name in ("W1", "b1", "W2", "b2", "W3", "b3"):
        assert _rel(dev_p[name], ref_p[name]) < 2e-3, name


def test_zero_output_layer_is_block_jacobi(gba, batch):
    """A fresh network (zero last layer) reproduces plain block-Jacobi exactly."""
    _, dev = batch
    m = gba.Mlp(seed=3, capacity=64)
    loss, base = m.loss_grad(*(dev[k].data_ptr() for k in ("f", "S", "L", "g", "x")), 40)
    assert loss == pytest.approx(base, rel=1e-12)


def test_adam_step_matches_reference_update(gba, batch, mlp_oracle):
    _, dev = batch
    m = gba.Mlp(capacity=64)
    p0 = _random_params(gba, mlp_oracle, 4)
    m.set_params(p0)
    m.loss_grad(*(dev[k].data_ptr() for k in ("f", "S", "L", "g", "x")), 40)
    g = m.grads().astype(np.float64)
    m.adam_step(1e-2, 0.9, 0.999, 1e-8)
    mh = 0.1 * g / (1 - 0.9)
    vh = 0.001 * g * g / (1 - 0.999)
    expect = p0 - 1e-2 * mh / (np.sqrt(vh) + 1e-8)
    assert _rel(m.params(), expect) < 1e-5


def test_training_reduces_loss(gba, batch):
    _, dev = batch
    m = gba.Mlp(seed=5, capacity=64)
    ptrs = [dev[k].data_ptr() for k in ("f", "S", "L", "g", "x")]
    l0, base = m.loss_grad(*ptrs, 40)
    for _ in range(300):
        m.loss_grad(*ptrs, 40)
        m.adam_step(3e-3)
    l1, _ = m.loss_grad(*ptrs, 40)
    assert l1 < 0.9 * l0


@pytest.mark.skipif(not MODEL.exists(), reason="trained model not present")
def test_trained_model_beats_block_jacobi_held_out():
    report = json.loads(MODEL.with_suffix(".json").read_text())
    assert report["held_out_loss"] < report["held_out_block_jacobi_loss"]


@pytest.mark.skipif(not MODEL.exists(), reason="trained model not present")
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


def test_learned_lm_reaches_oracle_cost_and_reports_gain(gba, oracle):
    """Workload-1 solve with the learned preconditioner: same accuracy bar as
    the mixed form (0.1% of the FP64 oracle), and the PCG work of both forms."""
    prob = gba.synthetic(1)
    ref, _, _ = oracle.solve(prob, max_iterations=20)
    mixed = gba.solve(prob.copy(), max_iterations=20, form="mixed")
    learned = gba.solve(prob.copy(), max_iterations=20, form="learned", model_path=str(MODEL))
    assert learned.anomalies == 0
    assert learned.final_cost <= ref["final_cost"] * (1 + 1e-3)
    print(f"PCG iterations: block-Jacobi {mixed.pcg_iterations}, learned {learned.pcg_iterations}")
