"""Ragged and degenerate problems through the C ABI, against the oracle.

The reference solver (src/lm.cu:371-724) has no special case for parameters
that no observation references: their normal-equation blocks are zero, the
damping lambda * max(diag, 1e-12) alone makes them SPD, and their step is
zero. Covered here: an unobserved camera and an unobserved point, points seen
by a single observation, a camera seen by a single observation, observations
in arbitrary (unsorted) order, and the empty problem (rejected, as the
reference reader rejects it: bal_reader.cpp:74). Tolerances as in the other
parity tests: the plain form's cost trajectory 1e-9 relative, the mixed
form's final cost within 0.1% of the oracle's.
"""
import numpy as np
import pytest

from conftest import PKG, rel_err

MODEL = PKG / "models" / "coarse_mlp.bin"


def _ragged(gba):
    base = gba.synthetic_custom(6, 300, 2, 5, 1.4, seed=31)
    C, P = base.num_cameras, base.num_points
    oc, op = base.obs_camera.copy(), base.obs_point.copy()
    px = base.obs_pixel.reshape(-1, 2).copy()
    keep = np.ones(oc.size, bool)
    for p in range(10):  # points 0..9 keep one observation
        keep[np.flatnonzero(op == p)[1:]] = False
    cam_last = np.flatnonzero((oc == C - 1) & keep)
    keep[cam_last[1:]] = False  # the last camera keeps one observation
    oc, op, px = oc[keep], op[keep], px[keep]
    perm = np.random.default_rng(5).permutation(oc.size)  # arbitrary observation order
    oc, op, px = oc[perm], op[perm], px[perm]
    cams = np.concatenate([base.cameras, base.cameras[:9]])  # camera C: unobserved
    pts = np.concatenate([base.points, [0.1, -0.2, 5.0]])    # point P: unobserved
    prob = gba.BALProblem(cams, pts, np.ascontiguousarray(oc, np.int32), np.ascontiguousarray(op, np.int32),
                          np.ascontiguousarray(px.ravel()))
    assert prob.num_cameras == C + 1 and prob.num_points == P + 1
    assert np.sum(prob.obs_camera == C - 1) == 1 and np.sum(prob.obs_point == 0) == 1
    return prob


def test_empty_problem_is_rejected(gba):
    """No observations (or no cameras / points): status 1 before any device work."""
    empty = gba.BALProblem(np.zeros(9), np.zeros(3), np.zeros(0, np.int32), np.zeros(0, np.int32), np.zeros(0))
    for form in ("plain", "mixed"):
        with pytest.raises(gba.GbaError) as e:
            gba.solve(empty, form=form)
        assert e.value.status == 1
    with pytest.raises(gba.GbaError):
        gba.Solver(empty, "mixed")


@pytest.mark.gpu
def test_ragged_plain_trajectory_matches_oracle(gba, oracle):
    prob = _ragged(gba)
    ref, ref_cams, ref_pts = oracle.solve(prob, max_iterations=10)
    run = prob.copy()
    res = gba.solve(run, max_iterations=10)
    reader = gba.total_squared_error(prob) / 2
    assert abs(res.initial_cost - reader) <= 1e-9 * max(1.0, reader)
    assert res.anomalies == 0
    assert res.iterations == ref["iterations"]
    t_dev, t_ref = np.array(res.trajectory), np.array(ref["trajectory"])
    assert t_dev.shape == t_ref.shape
    assert np.max(np.abs(t_dev - t_ref) / t_ref) < 1e-9
    assert rel_err(run.cameras, ref_cams) < 1e-6
    # unobserved parameters do not move
    assert np.array_equal(run.cameras[-9:], prob.cameras[-9:])
    assert np.array_equal(run.points[-3:], prob.points[-3:])


@pytest.mark.gpu
@pytest.mark.parametrize("form", ["mixed", "learned"])
def test_ragged_mixed_reaches_oracle_cost(gba, oracle, form):
    prob = _ragged(gba)
    ref, _, _ = oracle.solve(prob, max_iterations=15)
    run = prob.copy()
    opts = dict(max_iterations=15, form=form)
    if form == "learned":
        if not MODEL.exists():
            pytest.skip("trained model not present")
        opts["model_path"] = str(MODEL)
    res = gba.solve(run, **opts)
    assert res.anomalies == 0
    assert res.final_cost <= ref["final_cost"] * (1 + 1e-3)
    assert np.array_equal(run.cameras[-9:], prob.cameras[-9:])
    assert np.array_equal(run.points[-3:], prob.points[-3:])


@pytest.mark.gpu
@pytest.mark.parametrize("form", ["plain", "mixed"])
def test_non_spd_point_blocks_reject_every_trial(gba, form):
    """A negative damping makes every damped point block non-SPD: each trial is
    rejected before its step is taken (reference semantics: a non-SPD V block
    rejects the trial), lambda stays negative, and after max_inner_trials
    rejections the solve ends in FAILURE at the initial cost."""
    prob = gba.synthetic_custom(6, 300, 2, 5, 1.4, seed=31)
    run = prob.copy()
    res = gba.solve(run, form=form, initial_lambda=-1.5, max_inner_trials=3, max_iterations=2)
    assert res.termination == "FAILURE"
    assert res.iterations == 0 and res.trials == 3
    assert res.final_cost == res.initial_cost
    assert np.array_equal(run.cameras, prob.cameras) and np.array_equal(run.points, prob.points)


def test_oversized_problem_is_rejected(gba):
    """Sizes past the solver's 32-bit index range are refused up front (status 1),
    before any array is read or any device work starts: the arrays here are
    tiny, only the counts are large."""
    lib = gba.lib
    import ctypes as C
    one = np.zeros(9)
    idx = np.zeros(1, np.int32)
    for c, p, e in ((1, 400_000_000, 1), (1, 1, 1_100_000_000)):
        rc = lib.gba_solver_create(c, p, e, one.ctypes.data_as(C.POINTER(C.c_double)),
                                   one.ctypes.data_as(C.POINTER(C.c_double)), idx.ctypes.data_as(C.POINTER(C.c_int)),
                                   idx.ctypes.data_as(C.POINTER(C.c_int)), one.ctypes.data_as(C.POINTER(C.c_double)),
                                   0, None, C.byref(C.c_void_p()))
        assert rc == 1, rc
