"""ORACLE (test infrastructure only): CPU FP64 restatement of the learned
block-Jacobi MLP (forward, per-camera loss, backward) used to check the GPU
training kernels. It has no reference counterpart (the reference has no
iterative solver); its loss gradient is itself pinned by central finite
differences in the tests.

Layout of the flat parameter vector (FP32 masters): W1[128x64] b1[128]
W2[128x128] b2[128] W3[48x128] b3[48]. With emulate_bf16=True, GEMM operands
are rounded to BF16 exactly where the GPU kernels round them (weights and the
activation / gradient operand of every GEMM), and sums are exact (FP64), so the
GPU result differs only by its FP32 accumulation order.
"""
from __future__ import annotations

import numpy as np

IN, H, OUT = 64, 128, 48
USED_OUT = 45
SIZES = [("W1", (H, IN)), ("b1", (H,)), ("W2", (H, H)), ("b2", (H,)), ("W3", (OUT, H)), ("b3", (OUT,))]
N_PARAMS = sum(int(np.prod(s)) for _, s in SIZES)


def unpack(flat):
    out, o = {}, 0
    for name, shape in SIZES:
        n = int(np.prod(shape))
        out[name] = np.asarray(flat[o:o + n], np.float64).reshape(shape)
        o += n
    return out


def pack(d):
    return np.concatenate([np.asarray(d[name], np.float64).ravel() for name, _ in SIZES])


def bf16(a):
    """Round-to-nearest-even to bfloat16 (returned as float64)."""
    f = np.ascontiguousarray(np.asarray(a, np.float32))
    u = f.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def tri_index():
    return [(i, j) for i in range(9) for j in range(i + 1)]


TRI = tri_index()


def unpack_lower(v):
    L = np.zeros((9, 9))
    for k, (i, j) in enumerate(TRI):
        L[i, j] = v[k]
    return L


def build_F(o45):
    F = np.zeros((9, 9))
    th = np.tanh(o45)
    for k, (i, j) in enumerate(TRI):
        F[i, j] = np.exp(0.5 * th[k]) if i == j else 0.5 * th[k]
    return F, th


def sample_loss(o45, Shat45, Lhat45, g, x):
    """Loss of one camera: (y - x)^T S (y - x) / (x^T S x), y = (L F F^T L^T)^-1 g."""
    L = unpack_lower(Lhat45)
    S = unpack_lower(Shat45)
    S = S + np.tril(S, -1).T
    F, _ = build_F(o45)
    Lt = L @ F
    y = np.linalg.solve(Lt @ Lt.T, g)
    e = y - x
    return float(e @ S @ e / (x @ S @ x))


def sample_loss_grad(o45, Shat45, Lhat45, g, x):
    """Analytic gradient of sample_loss w.r.t. the 45 outputs (rank-2 form)."""
    L = unpack_lower(Lhat45)
    S = unpack_lower(Shat45)
    S = S + np.tril(S, -1).T
    F, th = build_F(o45)
    Lt = L @ F
    A = Lt @ Lt.T
    y = np.linalg.solve(A, g)
    den = x @ S @ x
    gy = 2 * S @ (y - x) / den
    z = np.linalg.solve(A, gy)
    a, b = Lt.T @ y, Lt.T @ z
    c, d = L.T @ z, L.T @ y
    out = np.zeros(45)
    for k, (i, j) in enumerate(TRI):
        dF = -(c[i] * a[j] + d[i] * b[j])
        dt = 0.5 * (1 - th[k] ** 2)
        out[k] = dF * F[i, i] * dt if i == j else dF * dt
    return out


def _rounding(emulate):
    """Operand rounding (BF16) and storage rounding (FP32) of the GPU kernels,
    or identities for the pure FP64 reference."""
    if emulate:
        return bf16, (lambda v: np.asarray(v, np.float32).astype(np.float64))
    ident = lambda v: np.asarray(v, np.float64)  # noqa: E731
    return ident, ident


def forward(flat, feat, emulate_bf16=True):
    p = unpack(flat)
    r, f32 = _rounding(emulate_bf16)
    X = np.asarray(feat, np.float64)
    h1 = f32(np.maximum(r(X) @ r(p["W1"]).T + p["b1"], 0))
    h2 = f32(np.maximum(r(h1) @ r(p["W2"]).T + p["b2"], 0))
    o = r(h2) @ r(p["W3"]).T + p["b3"]
    return o, (X, h1, h2)


def loss_and_grads(flat, feat, Shat, Lhat, g, x, emulate_bf16=True):
    """Mean loss over the batch, baseline (F = I) mean loss, and the flat gradient."""
    p = unpack(flat)
    r, f32 = _rounding(emulate_bf16)
    o, (X, h1, h2) = forward(flat, feat, emulate_bf16)
    o = f32(o)
    B = X.shape[0]
    dO = np.zeros((B, OUT))
    losses, base = [], []
    for b in range(B):
        losses.append(sample_loss(o[b, :USED_OUT], Shat[b], Lhat[b], g[b], x[b]))
        base.append(sample_loss(np.zeros(USED_OUT), Shat[b], Lhat[b], g[b], x[b]))  # o = 0 -> F = I
        dO[b, :USED_OUT] = sample_loss_grad(o[b, :USED_OUT], Shat[b], Lhat[b], g[b], x[b]) / B
    dO = f32(dO)
    grads = {}
    grads["W3"] = r(dO).T @ r(h2)
    grads["b3"] = dO.sum(0)
    dh2 = (r(dO) @ r(p["W3"])) * (h2 > 0)
    dh2 = f32(dh2)
    grads["W2"] = r(dh2).T @ r(h1)
    grads["b2"] = dh2.sum(0)
    dh1 = (r(dh2) @ r(p["W2"])) * (h1 > 0)
    dh1 = f32(dh1)
    grads["W1"] = r(dh1).T @ r(X)
    grads["b1"] = dh1.sum(0)
    return float(np.mean(losses)), float(np.mean(base)), pack(grads)


def scaled_sample(Scc, g_c, x_c):
    """Jacobi-scaled block quantities: S^ = D^-1/2 S D^-1/2, its Cholesky factor,
    g^ = D^-1/2 g, x^ = D^1/2 x (packed lower for the matrices)."""
    d = np.sqrt(np.diag(Scc))
    Sh = Scc / np.outer(d, d)
    Lh = np.linalg.cholesky(Sh)
    pk = lambda M: np.array([M[i, j] for (i, j) in TRI])  # noqa: E731
    return pk(Sh), pk(Lh), g_c / d, x_c * d
