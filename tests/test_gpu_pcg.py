"""GPU parity of the PCG solver and the shared radial distortion (the large robust workload's
solver, family 4) against the CPU oracle running the same algorithm (block-Jacobi PCG on the
reduced system, convergence tested every 4 iterations).

FP64: final cost within 1e-6 relative of the oracle.  Mixed precision (FP32 Jacobians and
reduced-camera products): the robust problem is still descending ~1e-4 per iteration after 15
iterations, so FP32 rounding of the steps moves the end point along the descent; the bar is that
mixed ends no more than 1e-6 above the FP64 oracle's cost (the same final cost or better) and
within 1e-5 of it either way.

Both forms of the reduced system the grid engine's PCG multiplies by are checked: the explicit
block-sparse S (the default) and the implicit products through the per-observation records
(chosen when the pair lists would be long); NAVBA_PCG_FORM selects one."""
import numpy as np
import pytest

from nav24_gb300 import abi
from nav24_gb300.synth import Synth, workload_options
from oracle import oracle

pytestmark = pytest.mark.gpu


def rel(a, b):
    return abs(a - b) / abs(b)


@pytest.fixture(params=["explicit", "implicit"])
def pcg_form(request, monkeypatch):
    monkeypatch.setenv("NAVBA_PCG_FORM", request.param)
    return request.param


def test_pcg_without_distortion_matches_oracle(ctx, pcg_form):
    p = Synth(1, n_cams=40, n_points=3000, seed=5).window(0)
    o = abi.default_options(iterations=10, robust=1, huber_delta=2.0, solver=abi.SOLVER_PCG,
                            pcg_tolerance=1e-10, pcg_max_iterations=400)
    g = ctx.solve(p, o)
    r = oracle.solve(p, o, n_threads=8)
    assert g.status == abi.OK and g.stats["pcg_iterations_total"] > 0
    assert rel(g.stats["final_cost"], r.stats["final_cost"]) < 1e-6


@pytest.mark.parametrize("precision", [abi.FP64, abi.MIXED])
def test_pcg_with_distortion_matches_oracle(ctx, pcg_form, precision):
    s = Synth(4, n_cams=60, n_points=6000, seed=8)
    p = s.window(0)
    o = workload_options(4)
    o.iterations = 15
    r = oracle.solve(p, o, n_threads=8)
    o.precision = precision
    g = ctx.solve(p, o)
    assert g.status == abi.OK
    if precision == abi.FP64:
        assert rel(g.stats["final_cost"], r.stats["final_cost"]) < 1e-6
    else:
        assert g.stats["final_cost"] <= r.stats["final_cost"] * (1 + 1e-6)
        assert rel(g.stats["final_cost"], r.stats["final_cost"]) < 1e-5
    assert abs(g.intrinsics[4] - r.intrinsics[4]) < 1e-5 and abs(g.intrinsics[5] - r.intrinsics[5]) < 1e-5
    # the radial factor d(r) = 1 + k1 r^2 + k2 r^4 over the image (r^2 <= 0.64) is recovered
    r2 = np.linspace(0.0, 0.64, 65)
    dd = lambda k: k[4] * r2 + k[5] * r2 * r2
    assert np.max(np.abs(dd(g.intrinsics) - dd(s.intrinsics))) < 2e-3


@pytest.mark.parametrize("precision", [abi.FP64, abi.MIXED])
def test_pcg_forms_agree_and_repeat_bitwise(ctx, monkeypatch, precision):
    """The explicit and implicit reduced systems are the same S: the two solves differ only by the
    rounding of the products (FP64: 1e-9 relative on the final cost, the same CG iteration count
    within a few; mixed: 1e-5).  Each form repeats bit for bit (fixed summation orders)."""
    p = Synth(4, n_cams=60, n_points=6000, seed=8).window(0)
    o = workload_options(4)
    o.iterations = 12
    o.precision = precision
    res = {}
    for f in ("explicit", "implicit"):
        monkeypatch.setenv("NAVBA_PCG_FORM", f)
        a, b = ctx.solve(p, o), ctx.solve(p, o)
        assert a.status == abi.OK and b.status == abi.OK
        assert np.array_equal(a.cam_pose, b.cam_pose) and np.array_equal(a.points, b.points)
        assert a.stats["pcg_iterations_total"] == b.stats["pcg_iterations_total"]
        res[f] = a
    ce, ci = res["explicit"].stats["final_cost"], res["implicit"].stats["final_cost"]
    assert rel(ce, ci) < (1e-9 if precision == abi.FP64 else 1e-5)
    if precision == abi.FP64:
        ie, ii = res["explicit"].stats["pcg_iterations_total"], res["implicit"].stats["pcg_iterations_total"]
        assert abs(ie - ii) <= max(4, ii // 50)


@pytest.mark.parametrize("fixed", ["every_7th", "all"])
def test_pcg_with_fixed_cameras_matches_oracle(ctx, pcg_form, fixed):
    """Fixed cameras leave holes in the reduced system's block rows; with every camera fixed and the
    shared distortion free, the reduced system is the 2x2 k block alone (no camera rows)."""
    p = Synth(4, n_cams=60, n_points=6000, seed=8).window(0)
    f = np.zeros(p.n_cams, np.uint8)
    if fixed == "all":
        f[:] = 1
    else:
        f[::7] = 1
    p.cam_fixed = f
    o = workload_options(4)
    o.iterations = 6
    r = oracle.solve(p, o, n_threads=8)
    g = ctx.solve(p, o)
    assert g.status == abi.OK and g.stats["n_free_cams"] == int((f == 0).sum())
    assert rel(g.stats["final_cost"], r.stats["final_cost"]) < 1e-6
    assert abs(g.intrinsics[4] - r.intrinsics[4]) < 1e-5 and abs(g.intrinsics[5] - r.intrinsics[5]) < 1e-5
    gp, pp = g.cam_pose.reshape(-1, 12), p.cam_pose.reshape(-1, 12)
    assert np.allclose(gp[f == 1], pp[f == 1], rtol=0, atol=1e-12)  # fixed cameras do not move
