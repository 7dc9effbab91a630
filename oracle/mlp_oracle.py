"""ORACLE (test infrastructure only): CPU FP64 restatement of the learned
coarse-basis MLP (forward, and backward from a given gradient w.r.t. the
outputs) used to check the GPU training kernels. It has no reference
counterpart (the reference has no iterative solver).

Layout of the flat parameter vector (FP32 masters): W1[128x64] b1[128]
W2[128x128] b2[128] W3[96x128] b3[96]. With emulate_bf16=True, GEMM operands
are rounded to BF16 exactly where the GPU kernels round them (weights and the
activation / gradient operand of every GEMM), and sums are exact (FP64), so the
GPU result differs only by its FP32 accumulation order.
"""
from __future__ import annotations

import numpy as np

IN, H, OUT = 64, 128, 96
USED_IN, USED_OUT = 58, 81
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


def backward(flat, feat, dO, emulate_bf16=True):
    """Flat parameter gradient of a loss whose gradient w.r.t. the outputs is dO (B x 96)."""
    p = unpack(flat)
    r, f32 = _rounding(emulate_bf16)
    _, (X, h1, h2) = forward(flat, feat, emulate_bf16)
    dO = f32(np.asarray(dO, np.float64))
    grads = {}
    grads["W3"] = r(dO).T @ r(h2)
    grads["b3"] = dO.sum(0)
    dh2 = f32((r(dO) @ r(p["W3"])) * (h2 > 0))
    grads["W2"] = r(dh2).T @ r(h1)
    grads["b2"] = dh2.sum(0)
    dh1 = f32((r(dh2) @ r(p["W2"])) * (h1 > 0))
    grads["W1"] = r(dh1).T @ r(X)
    grads["b1"] = dh1.sum(0)
    return pack(grads)


def coarse_basis(o, cams):
    """Z (9C x 9, column j of camera c's rows i at [9c + i, j]) from outputs o
    (C x 96): Z_c(i, j) = o[9 i + j] * unit_i, unit 1 except the focal row (f)."""
    C = o.shape[0]
    u = np.ones((C, 9))
    u[:, 6] = np.asarray(cams).reshape(C, 9)[:, 6]
    return (np.asarray(o, np.float64)[:, :81].reshape(C, 9, 9) * u[:, :, None]).reshape(9 * C, 9)
