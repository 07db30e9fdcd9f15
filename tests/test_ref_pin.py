"""The oracle and the GPU path against nav24's own edge code.

tests/golden/ref_edges.npz holds residuals, Jacobians and depth tests computed by the reference's
EdgeSE3ProjectXYZ (OptimizableTypes.hpp:102-113, OptimizableTypes.cpp:140-161), Calibration
(Calibration.cpp:235-247), Pinhole (Pinhole.cpp:30-36,70-80) and KannalaBrandt8
(KannalaBrandt8.cpp:80-107,195-226), compiled unmodified from the reference tree by
oracle/ref_build.py (generator: tests/golden/make_ref_vectors.py).

Bars: pinhole residuals and Jacobians 1e-12 relative for the oracle and 1e-10 for the GPU (FP64);
Kannala-Brandt 8: the oracle's reference-rounding mode 1e-12; the FP64 form (the oracle's default
and the GPU's), which evaluates the fisheye angles in FP64 where the reference's project rounds
them through atan2f and forms 3 k1 .. 9 k4 in float, within 1e-4 px of the reference's residuals
and 1e-8 of its Jacobians."""
from pathlib import Path

import numpy as np
import pytest

from nav24_gb300 import abi
from oracle import oracle

from ref_cases import CASES, sample

FIXTURE = Path(__file__).resolve().parent / "golden" / "ref_edges.npz"
PINHOLE = ["ring", "window", "eight", "behind"]


@pytest.fixture(scope="module")
def fix():
    return np.load(FIXTURE)


def rel(a, b):
    return np.max(np.abs(a - b)) / np.max(np.abs(b))


def _problem(name, fix):
    p = CASES[name]()
    assert p.n_obs == int(fix[f"{name}/n_obs"])
    idx = fix[f"{name}/idx"]
    assert np.array_equal(idx, sample(p.n_obs))
    return p, idx


def _depth_positive(p):
    P = p.cam_pose.reshape(-1, 3, 4)
    z = np.einsum("ij,ij->i", P[p.obs_cam, 2, :3], p.points[p.obs_point]) + P[p.obs_cam, 2, 3]
    return (z > 0).astype(np.uint8)


@pytest.mark.parametrize("name", PINHOLE)
def test_oracle_matches_reference_pinhole(fix, name):
    p, idx = _problem(name, fix)
    e, jc, jp, _ = oracle.linearize(p, abi.default_options())
    assert rel(e[idx], fix[f"{name}/e"]) < 1e-12
    assert rel(jc[idx], fix[f"{name}/jc"]) < 1e-12
    assert rel(jp[idx], fix[f"{name}/jp"]) < 1e-12


def test_oracle_matches_reference_kb8(fix):
    p, idx = _problem("kb8", fix)
    o = abi.default_options()
    e, jc, jp, _ = oracle.linearize(p, o, reference_rounding=True)
    assert rel(e[idx], fix["kb8/e"]) < 1e-12
    assert rel(jc[idx], fix["kb8/jc"]) < 1e-12
    assert rel(jp[idx], fix["kb8/jp"]) < 1e-12
    # the FP64 form: angles in FP64 (a documented deviation)
    e, jc, jp, _ = oracle.linearize(p, o)
    assert np.max(np.abs(e[idx] - fix["kb8/e"])) < 1e-4
    assert rel(jc[idx], fix["kb8/jc"]) < 1e-8 and rel(jp[idx], fix["kb8/jp"]) < 1e-8


@pytest.mark.parametrize("name", list(CASES))
def test_reference_depth_test(fix, name):
    """isDepthPositive is Z_c > 0 of the point in the camera."""
    p, idx = _problem(name, fix)
    assert np.array_equal(fix[f"{name}/depth_positive"], _depth_positive(p)[idx])


@pytest.mark.parametrize("name", list(CASES))
def test_fixture_regenerates_from_reference(fix, name):
    """Where the reference tree exists, its code still gives the committed vectors bit for bit."""
    from oracle import ref
    if ref.lib() is None:
        pytest.skip("the reference tree is absent on this host")
    p, idx = _problem(name, fix)
    e, jc, jp, dpos = ref.edges(p)
    for key, v in (("e", e), ("jc", jc), ("jp", jp), ("depth_positive", dpos)):
        assert np.array_equal(v[idx], fix[f"{name}/{key}"]), key


@pytest.mark.gpu
@pytest.mark.parametrize("name", PINHOLE + ["kb8"])
def test_gpu_linearize_matches_reference(ctx, fix, name):
    p, idx = _problem(name, fix)
    e, jc, jp, _ = ctx.linearize(p, abi.default_options())
    if name == "kb8":
        assert np.max(np.abs(e[idx] - fix["kb8/e"])) < 1e-4
        assert rel(jc[idx], fix["kb8/jc"]) < 1e-8 and rel(jp[idx], fix["kb8/jp"]) < 1e-8
    else:
        assert rel(e[idx], fix[f"{name}/e"]) < 1e-10
        assert rel(jc[idx], fix[f"{name}/jc"]) < 1e-10
        assert rel(jp[idx], fix[f"{name}/jp"]) < 1e-10


@pytest.mark.gpu
@pytest.mark.parametrize("solver", [abi.SOLVER_CHOLESKY, abi.SOLVER_PCG])
def test_gpu_depth_count_matches_reference(ctx, fix, solver):
    """nav_ba_result.n_depth_nonpositive counts the active edges whose isDepthPositive is false:
    at the initial state (0 iterations) it equals the reference's own depth tests of the 'behind'
    case, in the window engine (Cholesky) and the whole-GPU engine (PCG)."""
    p, idx = _problem("behind", fix)
    assert idx.size == p.n_obs  # every edge is in the fixture
    o = abi.default_options(iterations=0, solver=solver)
    g = ctx.solve(p, o)
    assert g.status == abi.OK
    assert g.stats["n_depth_nonpositive"] == int((fix["behind/depth_positive"] == 0).sum())
    r = oracle.solve(p, o)
    assert r.stats["n_depth_nonpositive"] == g.stats["n_depth_nonpositive"]


@pytest.mark.gpu
def test_gpu_depth_count_after_solve_matches_oracle(ctx):
    """After a solve the count is taken at the final state; on the ring workload every point ends in
    front of its cameras, in both precisions, as in the oracle."""
    from nav24_gb300.synth import Synth, workload_options
    p = Synth(0).window(0)
    r = oracle.solve(p, workload_options(0))
    for precision in (abi.FP64, abi.MIXED):
        o = workload_options(0)
        o.precision = precision
        g = ctx.solve(p, o)
        assert g.stats["n_depth_nonpositive"] == r.stats["n_depth_nonpositive"] == 0


@pytest.mark.gpu
def test_gpu_pose_depth_count(ctx, fix):
    """Motion-only problems report the observations behind the final pose (0 iterations: the
    reference's depth tests of the 'behind' case, camera by camera)."""
    p, _ = _problem("behind", fix)
    dpos = fix["behind/depth_positive"]
    probs, want = [], []
    for c in range(p.n_cams):
        sel = np.nonzero(p.obs_cam == c)[0]
        if sel.size == 0:
            continue
        probs.append(abi.PoseProblem(pose=p.cam_pose[c], points=p.points[p.obs_point[sel]], obs_uv=p.obs_uv[sel],
                                     intrinsics=p.intrinsics, camera_model=p.camera_model))
        want.append(int((dpos[sel] == 0).sum()))
    res = ctx.solve_pose_batched(probs, abi.default_options(iterations=0))
    assert [st["n_depth_nonpositive"] for _, st in res] == want
