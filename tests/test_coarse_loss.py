"""CPU: the learned coarse space's training loss (train_preconditioner.py).

The loss is the weighted share of the lowest eigenvectors of the
Jacobi-preconditioned reduced camera system that lies outside the span of the
network's basis; its closed-form gradient w.r.t. the network outputs is checked
against central finite differences, and its values at the two extremes (a
basis containing the eigenvectors, one orthogonal to them)."""
import numpy as np

from conftest import PKG  # noqa: F401  (puts the package on sys.path)
import train_preconditioner as tp


def _system(C=6, m=4, seed=0):
    rng = np.random.default_rng(seed)
    n = 9 * C
    V, _ = np.linalg.qr(rng.standard_normal((n, m)))
    Bl = np.tril(rng.standard_normal((C, 9, 9))) + 3 * np.eye(9)[None]
    cams = np.zeros((C, 9))
    cams[:, 6] = rng.uniform(400, 600, C)
    O = rng.standard_normal((C, 96)) * 0.1
    O[:, 81:] = 0.0
    return O, cams, Bl, V


def test_loss_gradient_matches_finite_differences():
    O, cams, Bl, V = _system()
    w = np.array([1.0, 2.0, 0.5, 1.0])
    loss, dO, _ = tp.coarse_loss_and_grad(O, cams, Bl, V, w)
    rng = np.random.default_rng(3)
    worst = 0.0
    for _ in range(40):
        c, k = rng.integers(O.shape[0]), rng.integers(81)
        h = 1e-6
        Op, Om = O.copy(), O.copy()
        Op[c, k] += h
        Om[c, k] -= h
        fd = (tp.coarse_loss_and_grad(Op, cams, Bl, V, w)[0] - tp.coarse_loss_and_grad(Om, cams, Bl, V, w)[0]) / (2 * h)
        worst = max(worst, abs(fd - dO[c, k]) / max(1e-6, np.max(np.abs(dO))))
    assert worst < 1e-6, worst
    assert np.all(dO[:, 81:] == 0.0)


def test_loss_extremes():
    O, cams, Bl, V = _system(C=5, m=3, seed=1)
    C = O.shape[0]
    # a basis whose span (after B^T) holds the eigenvectors: loss 0
    Zh = np.hstack([V, np.random.default_rng(2).standard_normal((9 * C, tp.K - V.shape[1]))])
    Z = np.linalg.solve(np.transpose(Bl, (0, 2, 1)), Zh.reshape(C, 9, tp.K))
    O2 = O.copy()
    O2[:, :81] = (Z / tp.units(cams)[:, :, None]).reshape(C, 81)
    loss, _, cap = tp.coarse_loss_and_grad(O2, cams, Bl, V)
    assert loss < 1e-12 and np.allclose(cap, 1.0)
    # a basis orthogonal to them: loss 1
    Q, _ = np.linalg.qr(np.hstack([V, np.random.default_rng(4).standard_normal((9 * C, tp.K))]))
    Z = np.linalg.solve(np.transpose(Bl, (0, 2, 1)), Q[:, V.shape[1]:V.shape[1] + tp.K].reshape(C, 9, tp.K))
    O3 = O.copy()
    O3[:, :81] = (Z / tp.units(cams)[:, :, None]).reshape(C, 81)
    loss, _, cap = tp.coarse_loss_and_grad(O3, cams, Bl, V)
    assert abs(loss - 1.0) < 1e-12 and np.allclose(cap, 0.0, atol=1e-12)
