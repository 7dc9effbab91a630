"""Test configuration: paths to the library binding and the oracle, the `gpu`
marker, and shared fixtures."""
import os
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
PKG = ROOT / "gpu-bundle-adjustment_gb300"
sys.path.insert(0, str(PKG))
sys.path.insert(0, str(ROOT / "oracle"))
GOLDEN = Path(__file__).resolve().parent / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the CUDA path through the C ABI")


def _ensure_built():
    sys.path.insert(0, str(PKG))
    import build as gba_build  # noqa: E402

    gba_build.build()


@pytest.fixture(scope="session")
def gba():
    _ensure_built()
    import gba_gb300

    return gba_gb300


@pytest.fixture(scope="session")
def oracle():
    import oracle as oracle_mod

    return oracle_mod


@pytest.fixture(scope="session")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def rel_err(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    scale = max(np.max(np.abs(b)), 1e-300)
    return float(np.max(np.abs(a - b)) / scale)


def implicit_system(s, prob, lam):
    """rhs and x -> S x of the mixed form's system, in numpy FP64 from the device's
    own FP32 Jacobian records and FP64 U, V, bc, bp (the system the refinement solves)."""
    C, P = prob.num_cameras, prob.num_points
    J = jacobian_rows(s).astype(np.float64)
    order = s.download("order")
    cam = prob.obs_camera[order]
    pt = prob.obs_point[order]
    Jc = J[:, :18].reshape(-1, 2, 9)
    Jp = J[:, 18:].reshape(-1, 2, 3)
    U = s.download("U").reshape(C, 9, 9)
    Ud = np.diagonal(U, axis1=1, axis2=2)
    Ul = U + lam * np.einsum("ci,ij->cij", np.where(Ud > 0, Ud, 1e-12), np.eye(9))
    Vp = s.download("V").reshape(P, 6)
    V = np.empty((P, 3, 3))
    for k, (i, j) in enumerate([(0, 0), (1, 0), (1, 1), (2, 0), (2, 1), (2, 2)]):
        V[:, i, j] = Vp[:, k]
        V[:, j, i] = Vp[:, k]
    for i in range(3):
        d = V[:, i, i].copy()
        V[:, i, i] += lam * np.where(d > 0, d, 1e-12)
    Vinv = np.linalg.inv(V)
    bc, bp = s.download("bc").reshape(C, 9), s.download("bp").reshape(P, 3)

    def point_step(dc):  # dp = V'^-1 (bp - sum_e W_e^T dc)
        t = np.einsum("sri,si->sr", Jc, dc.reshape(C, 9)[cam])
        g = np.zeros((P, 3))
        np.add.at(g, pt, np.einsum("srj,sr->sj", Jp, t))
        return np.einsum("pij,pj->pi", Vinv, bp - g).ravel()

    def back(g):  # g (P,3) -> sum over slots of Jc^T Jp Vinv g, per camera
        w = np.einsum("pij,pj->pi", Vinv, g)
        u = np.einsum("sij,sj->si", Jp, w[pt])
        out = np.zeros((C, 9))
        np.add.at(out, cam, np.einsum("sri,sr->si", Jc, u))
        return out

    rhs = (bc - back(bp)).ravel()

    def matvec(x):
        x = x.reshape(C, 9)
        t = np.einsum("sri,si->sr", Jc, x[cam])
        g = np.zeros((P, 3))
        np.add.at(g, pt, np.einsum("srj,sr->sj", Jp, t))
        return (np.einsum("cij,cj->ci", Ul, x) - back(g)).ravel()

    matvec.point_step = point_step
    return rhs, matvec


def shuffle_cameras(prob, seed):
    """The same problem with its cameras renumbered by a seeded permutation:
    returns (problem, new_index) with camera c of prob at new_index[c]."""
    rng = np.random.default_rng(seed)
    C = prob.num_cameras
    new_index = rng.permutation(C).astype(np.int32)
    cams = np.empty_like(prob.cameras).reshape(C, 9)
    cams[new_index] = prob.cameras.reshape(C, 9)
    out = prob.copy()
    out.cameras = cams.ravel()
    out.obs_camera = new_index[prob.obs_camera]
    return out, new_index


def jacobian_rows(s):
    """The mixed form's FP32 Jacobian rows as (E, 24) = [Jc (2 x 9 row-major), Jp
    (2 x 3)] per slot, from their device layout in component planes (Jc: four
    float4 planes and a float2 plane; Jp: a float4 and a float2 plane)."""
    E = s.dims()[2]
    a, b = s.download("Jc32"), s.download("Jp32")
    js = a.size // 18
    jc = np.hstack([a[:16 * js].reshape(4, js, 4).transpose(1, 0, 2).reshape(js, 16), a[16 * js:].reshape(js, 2)])
    jp = np.hstack([b[:4 * js].reshape(js, 4), b[4 * js:].reshape(js, 2)])
    return np.hstack([jc, jp])[:E]
