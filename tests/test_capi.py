"""CPU: the C-ABI library loads, exports every symbol include/gba_capi.h
declares, and its host-only entry points behave (no GPU compute here)."""
import re
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]


def _declared_symbols():
    text = (ROOT / "include" / "gba_capi.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(gba_[a-z0-9_]+)\s*\(", text)))


def test_header_symbols_exported(gba):
    import ctypes

    syms = _declared_symbols()
    assert len(syms) >= 30
    lib = ctypes.CDLL(str(gba.LIB_PATH))
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing
    # the Python binding covers every declared entry point
    assert set(syms) <= set(gba.EXPORTED), set(syms) - set(gba.EXPORTED)


def test_version_and_error_channel(gba):
    assert b"sm_103a" in gba.lib.gba_version()
    with pytest.raises(gba.GbaError) as ei:
        gba.load_bal("/nonexistent/problem.txt")
    assert "cannot open" in str(ei.value)


@pytest.mark.parametrize("workload,C,P,E_lo,E_hi", [(1, 16, 22000, 76000, 92000)])
def test_synthetic_workload_shapes(gba, workload, C, P, E_lo, E_hi):
    prob = gba.synthetic(workload)
    assert prob.num_cameras == C and prob.num_points == P
    assert E_lo <= prob.num_observations <= E_hi
    assert prob.obs_camera.min() >= 0 and prob.obs_camera.max() < C
    assert prob.obs_point.min() >= 0 and prob.obs_point.max() < P
    # camera-major order like the BAL files
    assert np.all(np.diff(prob.obs_camera) >= 0)
    # deterministic for a seed, different across seeds
    again = gba.synthetic(workload)
    np.testing.assert_array_equal(again.obs_pixel, prob.obs_pixel)
    other = gba.synthetic(workload, seed=99)
    assert other.num_observations != prob.num_observations or not np.array_equal(other.obs_pixel, prob.obs_pixel)


def test_synthetic_points_in_front_of_their_cameras(gba):
    prob, truth = gba.synthetic(1, with_truth=True)
    # residual of the truth at the observation must be the noise (~N(0,1) px)
    idx = np.arange(0, prob.num_observations, 97)
    res = np.array([gba.snavely_residual(truth.cameras[9 * prob.obs_camera[e]:9 * prob.obs_camera[e] + 9],
                                         truth.points[3 * prob.obs_point[e]:3 * prob.obs_point[e] + 3],
                                         prob.obs_pixel[2 * e:2 * e + 2]) for e in idx])
    assert 0.7 < np.std(res) < 1.3


def test_launch_bounds_generator_is_noise_free(gba):
    prob = gba.launch_bounds_problem(2000)
    assert prob.num_cameras == 8 and prob.num_observations == 4000
    assert list(prob.obs_camera[:4]) == [0, 1, 1, 2]
    # perturbation is live: the initial SSE is large
    assert gba.total_squared_error(prob) > 1.0


def test_options_defaults_mirror_reference(gba):
    o = gba.default_options()
    assert (o.max_iterations, o.initial_lambda, o.rel_decrease_tol, o.max_inner_trials, o.verbose) == (
        50, 1e-3, 1e-6, 16, 0)
