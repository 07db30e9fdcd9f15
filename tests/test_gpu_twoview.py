"""GPU parity of nav_ba_twoview_check (TwoViewReconstruction::Triangulate + CheckRT over every
hypothesis and match) against the numpy restatement: the same matches pass every check (the
decisions agree except where a quantity sits within rounding of a threshold), the triangulated points
agree to 1e-8 relative, nGood and the parallax statistic match, and the true hypothesis wins."""
import numpy as np
import pytest

from oracle import twoview as ref
from twoview_util import K, scene

pytestmark = pytest.mark.gpu

TH2 = 4.0 * 1.0  # 4 sigma^2 with sigma = 1 px
MINPC = 0.99998  # cos of the minimum parallax (about 0.36 deg)


def near_threshold(q, i, th2, minpc):
    """Whether match i sits within rounding of one of CheckRT's thresholds: a squared reprojection
    error within 1e-6 of th2 (relative), the cos-parallax within 1e-9 of its minimum, or a depth
    within 1e-9 of zero relative to the point's distance (the GPU's DLT point agrees with the
    restatement's to 1e-8 relative, so only such matches can be decided differently)."""
    return bool(abs(q["err1"][i] - th2) <= 1e-6 * th2 or abs(q["err2"][i] - th2) <= 1e-6 * th2 or
                abs(q["cos"][i] - minpc) <= 1e-9 or abs(q["z1"][i]) <= 1e-9 * q["r1"][i] or
                abs(q["z2"][i]) <= 1e-9 * q["r2"][i])


def test_twoview_matches_oracle(ctx):
    kp1, kp2, inl, Rs, ts, X = scene()
    g = ctx.twoview_check(K, kp1, kp2, Rs, ts, TH2, MINPC, 50, inlier=inl)
    for h in range(len(Rs)):
        q = {}
        pts, tri, good, ngood, par = ref.check_rt(K, kp1, kp2, Rs[h], ts[h], TH2, MINPC, 50, inl, quantities=q)
        assert abs(int(g["n_good"][h]) - ngood) <= 2
        assert np.sum(g["triangulated"][h] != tri) <= 2
        assert np.sum(g["good"][h] != good) <= 2
        # every decision that differs sits within rounding of a threshold
        for i in np.nonzero((g["triangulated"][h] != tri) | (g["good"][h] != good))[0]:
            assert near_threshold(q, i, TH2, MINPC), (h, i, {k: v[i] for k, v in q.items()})
        both = tri & g["triangulated"][h]
        if both.any():
            err = np.abs(g["points"][h][both] - pts[both]) / np.abs(pts[both]).max(axis=1, keepdims=True)
            assert err.max() < 1e-8
        if ngood > 60:
            assert abs(g["parallax_deg"][h] - par) < 1e-6
    assert int(np.argmax(g["n_good"])) == 0  # the true relative pose has the most points in front


def test_twoview_noise_free_recovers_points(ctx):
    kp1, kp2, inl, Rs, ts, X = scene(n=300, seed=11)
    from twoview_util import project
    kp1 = project(X)
    kp2 = project(X @ Rs[0].T + ts[0])
    g = ctx.twoview_check(K, kp1, kp2, Rs[:1], ts[:1], TH2, MINPC, 50)
    assert g["triangulated"][0].all()
    assert np.max(np.abs(g["points"][0] - X)) < 1e-8
