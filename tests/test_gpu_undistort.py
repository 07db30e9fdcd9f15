"""GPU parity of nav_ba_undistort_points (cv::undistortPoints with R = I, P = K, as nav24's
PinholeRadTan::UndistortKeyPoints calls it) against the numpy restatement: 1e-12 px for the default
5 iterations; with enough iterations the forward model maps the result back onto the input."""
import numpy as np
import pytest

from oracle import undistort as ref

pytestmark = pytest.mark.gpu

K = np.array([458.654, 457.296, 367.215, 248.375])     # a typical VGA radial-tangential calibration
D = np.array([-0.28340811, 0.07395907, 0.00019359, 1.76187114e-05])


def keypoints(n=20000, seed=4):
    rng = np.random.default_rng(seed)
    return np.stack([rng.uniform(0, 752, n), rng.uniform(0, 480, n)], axis=1)


@pytest.mark.parametrize("iters", [0, 1, 5, 30])
def test_undistort_matches_oracle(ctx, iters):
    uv = keypoints()
    g = ctx.undistort_points(K, D, uv, iters)
    r = ref.undistort(K, D, uv, iters)
    assert np.max(np.abs(g - r)) < 1e-9


def test_undistort_round_trip(ctx):
    uv = keypoints(5000)
    und = ctx.undistort_points(K, D, uv, 50)
    inside = np.all((und > -200) & (und < 1000), axis=1)   # the fixed point exists away from the far corners
    back = ref.distort(K, D, und[inside])
    assert np.max(np.abs(back - uv[inside])) < 1e-6


def test_undistort_empty(ctx):
    assert ctx.undistort_points(K, D, np.zeros((0, 2))).shape == (0, 2)
