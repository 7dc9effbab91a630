"""GPU: the plain form's band layout of S (cameras renumbered by reverse
Cuthill-McKee, S and its Cholesky factor kept as a band) against the oracle.

The band layout computes the reference's dense step (src/lm.cu:598-604: Eigen
LLT of the full (9C)^2 matrix) with fewer flops; it must give the same step:
  - band Cholesky / solve kernels vs numpy on random SPD band matrices, 1e-12 / 1e-10;
  - the ordering equals the oracle's (oracle/band_oracle.py) exactly;
  - the assembled diagonal blocks equal the dense layout's bit for bit;
  - the Schur step dc within 1e-9 of the oracle's FP64 step and of the dense layout's;
  - whole LM solves: per-iteration cost within 1e-9 of the oracle, same iterations.
"""
import time

import numpy as np
import pytest

from conftest import rel_err, shuffle_cameras

pytestmark = pytest.mark.gpu


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _band_spd(n, bt, seed):
    """Random SPD matrix whose nonzeros lie within bt 64-row tiles below each diagonal tile."""
    rng = np.random.default_rng(seed)
    ti = np.arange(n) // 64
    mask = np.abs(np.subtract.outer(ti, ti)) <= bt
    M = rng.normal(size=(n, n)) * mask
    A = (M + M.T) / 2
    A += (np.abs(A).sum(axis=1).max() + 1.0) * np.eye(n)  # diagonally dominant
    return A


@pytest.mark.parametrize("n,bt", [(640, 2), (640, 0), (448, 6), (1280, 3), (192, 1)])
def test_band_potrf_potrs_match_numpy(gba, torch_cuda, n, bt):
    import band_oracle as bo

    torch = torch_cuda
    ldb = (bt + 2) * 64
    A = _band_spd(n, bt, seed=n + bt)
    dA = _dev(torch, bo.to_band(A, ldb))
    info = torch.zeros(1, dtype=torch.int32, device="cuda")
    gba.band_potrf(dA.data_ptr(), n, ldb, bt, info.data_ptr())
    torch.cuda.synchronize()
    assert int(info.item()) == 0
    L = bo.from_band(dA.cpu().numpy(), n, ldb, rows=min(ldb - 64, n))
    assert rel_err(L, np.linalg.cholesky(A)) < 1e-12
    b = np.random.default_rng(1).normal(size=n)
    db = _dev(torch, b)
    gba.band_potrs(dA.data_ptr(), n, ldb, bt, db.data_ptr(), info.data_ptr())
    torch.cuda.synchronize()
    assert rel_err(db.cpu().numpy(), np.linalg.solve(A, b)) < 1e-10


def test_band_potrf_reports_failed_column(gba, torch_cuda):
    import band_oracle as bo

    torch = torch_cuda
    n, bt = 320, 1
    A = 4.0 * np.eye(n)
    A[200, 200] = -1.0
    ldb = (bt + 2) * 64
    dA = _dev(torch, bo.to_band(A, ldb))
    info = torch.zeros(1, dtype=torch.int32, device="cuda")
    gba.band_potrf(dA.data_ptr(), n, ldb, bt, info.data_ptr())
    torch.cuda.synchronize()
    assert int(info.item()) == 201


@pytest.fixture(scope="module")
def local(gba):
    return gba.synthetic_local(300, 30000, 2, 8, 1.5, 10, seed=3)


@pytest.fixture(scope="module")
def shuffled(local):
    return shuffle_cameras(local, seed=5)[0]


def _step(gba, prob, layout, lam):
    with gba.Solver(prob, "plain") as s:
        s.set_schur_layout(layout)
        gba.solver_set_harvest(s, True)
        s.accumulate()
        assert s.damp_invert_v(lam) == 0
        assert s.schur_dense(lam) == 0
        ldb, bt, perm = s.schur_band()
        out = dict(dc=s.download("dc"), rhs=s.download("rhs")[:9 * prob.num_cameras], Sdiag=s.download("Sdiag"),
                   ldb=ldb, bt=bt, perm=perm)
        out["denom"] = s.back_substitute(lam)
        out["dp"] = s.download("dp")
    return out


@pytest.mark.parametrize("which", ["local", "shuffled"])
def test_band_schur_step_matches_oracle_and_dense(gba, oracle, request, which):
    import band_oracle as bo

    prob = request.getfixturevalue(which)
    lam = 3e-3
    C = prob.num_cameras
    plan = bo.band_plan(C, *bo.camera_graph(prob))
    band = _step(gba, prob, "auto", lam)
    dense = _step(gba, prob, "dense", lam)
    assert dense["ldb"] == 0 and dense["perm"] is None
    assert band["ldb"] == plan["ldb"] and band["bt"] == plan["bt"]
    assert np.array_equal(band["perm"], plan["perm"])
    if which == "shuffled":
        assert not np.array_equal(plan["perm"], np.arange(C))
    assert np.array_equal(band["Sdiag"], dense["Sdiag"])  # same ordered sums, other place
    assert np.array_equal(band["rhs"], dense["rhs"])
    ref = oracle.schur_step(prob, lam, threads=2)
    assert ref["status"] == 0
    assert rel_err(band["dc"], ref["dc"]) < 1e-9
    assert rel_err(band["dc"], dense["dc"]) < 1e-10
    assert rel_err(band["dp"], ref["dp"]) < 1e-9
    assert abs(band["denom"] - ref["denom"]) <= 1e-9 * abs(ref["denom"])


def test_band_forced_on_dense_graph_matches_dense(gba):
    """The band layout forced on a random-covisibility problem (band = whole matrix)."""
    prob = gba.synthetic_custom(40, 3000, 2, 8, 1.6, seed=17)
    lam = 1e-3
    band = _step(gba, prob, "band", lam)
    dense = _step(gba, prob, "dense", lam)
    assert band["ldb"] > 0
    assert rel_err(band["dc"], dense["dc"]) < 1e-10


@pytest.mark.parametrize("which", ["local", "shuffled"])
def test_band_lm_trajectory_matches_oracle(gba, oracle, request, which):
    prob = request.getfixturevalue(which)
    ref, _, _ = oracle.solve(prob, max_iterations=15, threads=2)
    res = gba.solve(prob.copy(), max_iterations=15)
    assert res.schur_band_rows > 0
    assert res.anomalies == 0
    assert res.termination == ref["termination"] and res.iterations == ref["iterations"]
    t, r = np.array(res.trajectory), np.array(ref["trajectory"])
    assert t.shape == r.shape
    assert np.max(np.abs(t - r) / r) < 1e-9


def test_band_layout_faster_than_dense_and_same_step(gba):
    """800 cameras on a path (dense S: 7,232^2 doubles): one plain Schur step
    in the band layout against the dense one, after a warm-up step each."""
    prob = gba.synthetic_local(800, 80000, 2, 8, 1.5, 10, seed=8)
    lam = 1e-3
    secs, dcs = {}, {}
    for layout in ("dense", "band"):
        with gba.Solver(prob, "plain") as s:
            s.set_schur_layout(layout)
            s.accumulate()
            assert s.damp_invert_v(lam) == 0
            assert s.schur_dense(lam) == 0  # warm-up (allocates S, plans the band)
            t0 = time.perf_counter()
            for _ in range(3):
                assert s.schur_dense(lam) == 0
            secs[layout] = (time.perf_counter() - t0) / 3
            dcs[layout] = s.download("dc")
    print(f"Schur step, 800 cameras on a path: dense {secs['dense'] * 1e3:.2f} ms, band {secs['band'] * 1e3:.2f} ms")
    assert rel_err(dcs["band"], dcs["dense"]) < 1e-10
    assert secs["band"] * 3 < secs["dense"], secs
