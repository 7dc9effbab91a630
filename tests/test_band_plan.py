"""CPU: the local-covisibility generator and the band ordering oracle
(oracle/band_oracle.py) that the plain form's band layout is checked against."""
import numpy as np
import pytest

from conftest import shuffle_cameras


@pytest.fixture(scope="module")
def local(gba):
    return gba.synthetic_local(300, 30000, 2, 8, 1.5, 10, seed=3)


def test_local_generator_tracks_stay_in_window(gba, local):
    """Every track's cameras lie within 2 * window of each other, so the
    camera graph in the generator's order is a band of half-width <= 20."""
    import band_oracle as bo

    a, b = bo.camera_graph(local)
    assert len(a) > 0
    assert int(np.max(a - b)) <= 20
    assert local.num_observations > 2 * local.num_points
    again = gba.synthetic_local(300, 30000, 2, 8, 1.5, 10, seed=3)
    for x, y in zip(local.arrays(), again.arrays()):
        assert np.array_equal(x, y)


def test_local_generator_initial_cost_is_moderate(gba, local):
    """The perturbation moves camera centres, not translations: the initial
    cost per observation stays comparable to the global generator's."""
    sse = gba.total_squared_error(local)
    assert np.isfinite(sse) and sse / local.num_observations < 1e4


def test_rcm_recovers_band_of_shuffled_cameras(local):
    """Shuffled camera indices: the graph looks dense in the given order; the
    reverse Cuthill-McKee order brings it back to a narrow band."""
    import band_oracle as bo

    shuffled, _ = shuffle_cameras(local, seed=5)
    a, b = bo.camera_graph(shuffled)
    assert int(np.max(np.abs(a - b))) > 150
    plan = bo.band_plan(shuffled.num_cameras, a, b)
    assert sorted(plan["perm"].tolist()) == list(range(shuffled.num_cameras))
    assert plan["w"] <= 40, plan["w"]
    assert plan["ldb"] == (plan["bt"] + 2) * 64 and 9 * (plan["w"] + 1) <= (plan["bt"] + 1) * 64


def test_band_plan_keeps_given_order_when_narrower(local):
    import band_oracle as bo

    a, b = bo.camera_graph(local)
    plan = bo.band_plan(local.num_cameras, a, b)
    assert np.array_equal(plan["perm"], np.arange(local.num_cameras))
    assert plan["w"] == int(np.max(a - b))


def test_band_storage_round_trip():
    import band_oracle as bo

    rng = np.random.default_rng(0)
    n, ldb = 200, 70
    A = rng.normal(size=(n, n))
    A = np.tril(A) * (np.subtract.outer(np.arange(n), np.arange(n)) < ldb)
    assert np.array_equal(bo.from_band(bo.to_band(A, ldb), n, ldb), A)
