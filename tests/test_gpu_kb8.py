"""GPU parity of the Kannala-Brandt camera model (NAV_BA_CAM_KANNALA_BRANDT8) against the oracle:
residuals and Jacobians 1e-10 (FP64), final cost after a fixed number of LM iterations 1e-6 on the
window engine (FP64 and mixed), the whole-GPU engine and the motion-only engine."""
import numpy as np
import pytest

from nav24_gb300 import abi
from oracle import oracle

from kb8_util import kb8_problem

pytestmark = pytest.mark.gpu


def rel(a, b):
    return abs(a - b) / abs(b)


def test_kb8_linearize_matches_oracle(ctx):
    p = kb8_problem(n_cams=12, n_points=500)
    o = abi.default_options(robust=1, huber_delta=2.0)
    g = ctx.linearize(p, o)
    r = oracle.linearize(p, o)
    for a, b in zip(g, r):
        assert np.max(np.abs(a - b)) / np.max(np.abs(b)) < 1e-10


@pytest.mark.parametrize("precision", [abi.FP64, abi.MIXED])
def test_kb8_window_solve_matches_oracle(ctx, precision):
    p = kb8_problem(n_cams=16, n_points=1500)
    of = abi.default_options(iterations=8, robust=1, huber_delta=2.0)
    r = oracle.solve(p, of, n_threads=8)
    o = abi.default_options(iterations=8, robust=1, huber_delta=2.0, precision=precision)
    g = ctx.solve(p, o)
    assert g.status == abi.OK
    assert rel(g.stats["final_cost"], r.stats["final_cost"]) < 1e-6


def test_kb8_grid_solve_matches_oracle(ctx):
    p = kb8_problem(n_cams=40, n_points=3000)  # 39 free cameras: the whole-GPU engine
    o = abi.default_options(iterations=6, robust=1, huber_delta=2.0)
    r = oracle.solve(p, o, n_threads=8)
    g = ctx.solve(p, o)
    assert g.status == abi.OK
    assert rel(g.stats["final_cost"], r.stats["final_cost"]) < 1e-6


def test_kb8_pose_only_matches_oracle(ctx):
    p = kb8_problem(n_cams=12, n_points=800)
    c = p.n_cams - 1
    sel = np.nonzero(p.obs_cam == c)[0]
    pp = abi.PoseProblem(pose=p.cam_pose[c], points=p.points[p.obs_point[sel]], obs_uv=p.obs_uv[sel],
                         intrinsics=p.intrinsics, camera_model=p.camera_model)
    o = abi.default_options(iterations=10)
    (pose, st), = ctx.solve_pose_batched([pp], o)
    r = oracle.solve(pp.as_problem(), o)
    assert rel(st["final_cost"], r.stats["final_cost"]) < 1e-10
    assert np.max(np.abs(pose - r.cam_pose[0])) < 1e-9
