"""GPU parity tests: the CUDA path (through the C ABI) against the CPU oracle on the same inputs.

Tolerances (FP64 form): observation indexing and the reduced-system sparsity pattern bit-exact,
residuals/Jacobians/reduced system within 1e-10 relative, cost after a fixed number of LM
iterations within 1e-6 relative.  Mixed form: final cost within 1e-6 relative of the FP64
oracle."""
import json
from pathlib import Path

import numpy as np
import pytest

from nav24_gb300 import abi
from nav24_gb300.synth import Synth, workload_options
from oracle import oracle

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).resolve().parent / "golden"


def rel_err(a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    return np.max(np.abs(a - b)) / max(1e-300, np.max(np.abs(b)))


def ring():
    g = np.load(GOLDEN / "ring_fixture.npz")
    return abi.Problem(cam_pose=g["cam_pose"], points=g["points"], obs_uv=g["obs_uv"], obs_cam=g["obs_cam"],
                       obs_point=g["obs_point"], intrinsics=g["intrinsics"], cam_fixed=g["cam_fixed"])


@pytest.mark.parametrize("robust", [0, 1])
def test_linearize_fp64_matches_oracle(ctx, robust):
    p = ring()
    o = abi.default_options(robust=robust, huber_delta=2.0)
    ge, gjc, gjp, gw = ctx.linearize(p, o)
    oe, ojc, ojp, ow = oracle.linearize(p, o)
    assert rel_err(ge, oe) < 1e-10
    assert rel_err(gjc, ojc) < 1e-10
    assert rel_err(gjp, ojp) < 1e-10
    assert rel_err(gw, ow) < 1e-10


def test_linearize_known_answers(ctx):
    for case in json.loads((GOLDEN / "known_answer.json").read_text()):
        p = abi.Problem(cam_pose=np.array(case["pose12"]), points=np.array(case["X"]), obs_uv=np.array(case["z"]),
                        obs_cam=[0], obs_point=[0], intrinsics=np.array(case["intrinsics"]),
                        camera_model=case["model"])
        e, jc, jp, _ = ctx.linearize(p, abi.default_options())
        assert rel_err(e[0], case["e"]) < 1e-12
        assert rel_err(jc[0], case["jc"]) < 1e-12
        assert rel_err(jp[0], case["jp"]) < 1e-12


def test_linearize_mixed_close_to_fp64(ctx):
    p = ring()
    o = abi.default_options(precision=abi.MIXED)
    ge, gjc, gjp, _ = ctx.linearize(p, o)
    oe, ojc, ojp, _ = oracle.linearize(p, abi.default_options())
    assert rel_err(gjc, ojc) < 1e-5
    assert rel_err(gjp, ojp) < 1e-5
    assert np.max(np.abs(ge - oe)) < 1e-3  # pixels


@pytest.mark.parametrize("lam", [1e-3, 10.0])
def test_reduced_system_pattern_and_values(ctx, lam):
    for p in (ring(), Synth(2, n_windows=1, n_cams=12, n_points=600, seed=11).window(0)):
        o = abi.default_options()
        gS, gb, gidx = ctx.reduced_system(p, o, lam)
        oS, ob, oidx = oracle.reduced_system(p, o, lam)
        assert np.array_equal(gidx, oidx)
        nf = oS.shape[0] // 6
        gpat = np.array([[np.any(gS[6 * a:6 * a + 6, 6 * b:6 * b + 6] != 0) for b in range(nf)] for a in range(nf)])
        opat = np.array([[np.any(oS[6 * a:6 * a + 6, 6 * b:6 * b + 6] != 0) for b in range(nf)] for a in range(nf)])
        assert np.array_equal(gpat, opat)
        assert rel_err(gS, oS) < 1e-10
        assert rel_err(gb, ob) < 1e-10


def test_cost_matches_oracle(ctx):
    p = ring()
    for robust in (0, 1):
        o = abi.default_options(robust=robust, huber_delta=2.0)
        assert abs(ctx.cost(p, o) - oracle.cost(p, o)) / oracle.cost(p, o) < 1e-12


def test_solve_fp64_matches_oracle_ring(ctx):
    p = ring()
    o = workload_options(0)
    g = ctx.solve(p, o)
    r = oracle.solve(p, o)
    assert g.status == abi.OK
    assert abs(g.stats["initial_cost"] - r.stats["initial_cost"]) / r.stats["initial_cost"] < 1e-12
    assert abs(g.stats["final_cost"] - r.stats["final_cost"]) / r.stats["final_cost"] < 1e-6
    n = min(len(g.cost_trace), len(r.cost_trace))
    assert rel_err(g.cost_trace[:n], r.cost_trace[:n]) < 1e-6
    assert np.allclose(g.points, r.points, rtol=0, atol=1e-6)
    assert np.allclose(g.cam_pose, r.cam_pose, rtol=0, atol=1e-7)
    assert g.stats["n_free_cams"] == r.stats["n_free_cams"]
    assert g.stats["n_active_edges"] == r.stats["n_active_edges"]
    assert g.stats["n_schur_blocks"] == r.stats["n_schur_blocks"]


def test_solve_fp64_robust_window(ctx):
    p = Synth(2, n_windows=1, seed=21).window(0)
    o = abi.default_options(iterations=10, robust=1, huber_delta=2.0)
    g = ctx.solve(p, o)
    r = oracle.solve(p, o)
    assert abs(g.stats["final_cost"] - r.stats["final_cost"]) / r.stats["final_cost"] < 1e-6


def test_solve_mixed_reaches_fp64_cost(ctx):
    p = ring()
    o = workload_options(0)
    r = oracle.solve(p, o)
    om = workload_options(0, precision=abi.MIXED)
    om.iterations = 20
    g = ctx.solve(p, om)
    assert g.status == abi.OK
    assert abs(g.stats["final_cost"] - r.stats["final_cost"]) / r.stats["final_cost"] < 1e-6


def test_batched_windows_match_oracle_per_window(ctx):
    s = Synth(2, n_windows=24, seed=5)
    wins = s.windows()
    o = workload_options(2)
    gs = ctx.solve_batched(wins, o)
    for w, g in zip(wins, gs):
        r = oracle.solve(w, o)
        assert g.status == abi.OK
        assert abs(g.stats["final_cost"] - r.stats["final_cost"]) / r.stats["final_cost"] < 1e-6
        assert np.allclose(g.points, r.points, rtol=0, atol=1e-5)


@pytest.mark.parametrize("precision", [abi.FP64, abi.MIXED])
def test_pipelined_batch_equals_single_solves(ctx, precision):
    """A batch of >= 64 windows runs in parts pipelined across host and device; every window's
    result equals (bitwise) that of solving the window alone."""
    s = Synth(2, n_windows=96, seed=8)
    wins = s.windows()
    o = workload_options(2, precision=precision)
    gs = ctx.solve_batched(wins, o)
    assert len({g.stats["h2d_bytes"] for g in gs}) == 1  # the whole call's bytes in every result
    for i in [0, 23, 24, 47, 50, 71, 72, 95]:
        g1 = ctx.solve(wins[i], o)
        assert gs[i].status == g1.status == abi.OK
        assert gs[i].stats["final_cost"] == g1.stats["final_cost"]
        assert np.array_equal(gs[i].points, g1.points)
        assert np.array_equal(gs[i].cam_pose, g1.cam_pose)


def test_pipelined_batch_reports_first_bad_window(ctx):
    """An invalid window in a later part fails the call with its own index; nothing is written."""
    from nav24_gb300._lib import BAError
    s = Synth(2, n_windows=80, seed=9)
    wins = s.windows()
    wins[70] = wins[70].copy()
    wins[70].points[3, 1] = np.nan
    with pytest.raises(BAError) as ei:
        ctx.solve_batched(wins, workload_options(2))
    assert ei.value.status == abi.ERR_NONFINITE_INPUT
    assert "problem 70" in str(ei.value)
    # the context stays usable; an empty window inside a pipelined batch is passed through
    good = wins[:70]
    e = good[40]
    good[40] = abi.Problem(cam_pose=e.cam_pose, points=e.points, obs_uv=np.zeros((0, 2)), obs_cam=[], obs_point=[],
                           intrinsics=e.intrinsics)
    g = ctx.solve_batched(good, workload_options(2))
    assert g[40].status == abi.EMPTY and np.array_equal(g[40].points, e.points)
    assert all(r.status == abi.OK for i, r in enumerate(g) if i != 40)
    g1 = ctx.solve(good[39], workload_options(2))
    assert g[39].stats["final_cost"] == g1.stats["final_cost"]


@pytest.mark.parametrize("precision", [abi.FP64, abi.MIXED])
def test_batched_512_windows_match_oracle(ctx, precision):
    """The whole batched workload (512 windows of family 2, seed 1002, 10 LM iterations: the
    benchmark's batch) in one call, every window's final cost against the FP64 oracle's within
    1e-6 relative, in both precisions (the oracle runs one window per host thread)."""
    from concurrent.futures import ThreadPoolExecutor
    import os
    wins = Synth(2).windows()
    assert len(wins) == 512
    o = workload_options(2)
    with ThreadPoolExecutor(max(1, os.cpu_count() or 1)) as ex:
        ref = list(ex.map(lambda w: oracle.solve(w, o), wins))
    og = workload_options(2, precision=precision)
    gs = ctx.solve_batched(wins, og)
    worst = max(abs(g.stats["final_cost"] - r.stats["final_cost"]) / r.stats["final_cost"] for g, r in zip(gs, ref))
    assert all(g.status == abi.OK for g in gs)
    assert worst < 1e-6, worst
    if precision == abi.FP64:
        assert worst < 1e-12, worst
        assert all(g.stats["iterations_done"] == r.stats["iterations_done"] and
                   g.stats["trials_accepted"] == r.stats["trials_accepted"] for g, r in zip(gs, ref))


def test_batched_mixed_reaches_fp64_cost(ctx):
    s = Synth(2, n_windows=16, seed=6)
    wins = s.windows()
    o = workload_options(2)
    om = workload_options(2, precision=abi.MIXED)
    gs = ctx.solve_batched(wins, om)
    for w, g in zip(wins, gs):
        r = oracle.solve(w, o)
        assert abs(g.stats["final_cost"] - r.stats["final_cost"]) / r.stats["final_cost"] < 1e-6


def test_edge_cases(ctx):
    p = ring()
    o = workload_options(0)
    # fixed points and an all-fixed-camera problem
    q = p.copy()
    q.point_fixed = np.zeros(q.n_points, np.uint8)
    q.point_fixed[::3] = 1
    g, r = ctx.solve(q, o), oracle.solve(q, o)
    assert abs(g.stats["final_cost"] - r.stats["final_cost"]) / r.stats["final_cost"] < 1e-6
    assert np.array_equal(g.points[::3], q.points[::3])
    q = p.copy()
    q.cam_fixed = np.ones(q.n_cams, np.uint8)
    g, r = ctx.solve(q, o), oracle.solve(q, o)
    assert abs(g.stats["final_cost"] - r.stats["final_cost"]) / r.stats["final_cost"] < 1e-6
    # duplicate observations of a point by the same camera
    q = p.copy()
    q.obs_uv = np.concatenate([q.obs_uv, q.obs_uv[:50] + 0.5])
    q.obs_cam = np.concatenate([q.obs_cam, q.obs_cam[:50]])
    q.obs_point = np.concatenate([q.obs_point, q.obs_point[:50]])
    q.__post_init__()
    g, r = ctx.solve(q, o), oracle.solve(q, o)
    assert abs(g.stats["final_cost"] - r.stats["final_cost"]) / r.stats["final_cost"] < 1e-6
    # empty problem
    q = abi.Problem(cam_pose=p.cam_pose, points=p.points, obs_uv=np.zeros((0, 2)), obs_cam=[], obs_point=[],
                    intrinsics=p.intrinsics)
    g = ctx.solve(q, o)
    assert g.status == abi.EMPTY and np.array_equal(g.points, p.points)
    # invalid inputs are rejected on the host and leave outputs untouched
    q = p.copy()
    q.obs_uv[7, 0] = np.inf
    g = ctx.solve(q, o, raise_on_error=False)
    assert g.status == abi.ERR_NONFINITE_INPUT and not np.any(g.points)
    q = p.copy()
    q.obs_point[3] = -1
    assert ctx.solve(q, o, raise_on_error=False).status == abi.ERR_ARGUMENT


def test_prepare_run_fetch_equals_solve(ctx):
    p = ring()
    o = workload_options(0)
    g = ctx.solve(p, o)
    ctx.prepare(p, o)
    for _ in range(2):
        st = ctx.run(o)
        assert st["final_cost"] == g.stats["final_cost"]
    f = ctx.fetch(o)
    assert np.array_equal(f.points, g.points)
    assert np.array_equal(f.cam_pose, g.cam_pose)


def test_run_replays_captured_launch_and_follows_new_options(ctx):
    """nav_ba_run replays the launch captured at prepare time; a run with other LM options (same
    precision and iterations) launches with those.  (Runs share the shape tuned at prepare time, so
    they compare bitwise among themselves; against solves, which may run another shape, the mixed
    form's partial sums differ in the last bits.)"""
    import copy
    s = Synth(2, n_windows=8, seed=12)
    p = s.window(3)
    o = workload_options(2, precision=abi.MIXED)
    o2 = copy.copy(o)
    o2.tau = o.tau * 100.0
    o2.robust = 1 - o.robust
    g, g2 = ctx.solve(p, o), ctx.solve(p, o2)
    ctx.prepare(p, o)
    r1, r2, r3 = ctx.run(o), ctx.run(o2), ctx.run(o)
    assert r3["final_cost"] == r1["final_cost"]
    assert r2["final_cost"] != r1["final_cost"]
    assert abs(r1["final_cost"] - g.stats["final_cost"]) / g.stats["final_cost"] < 1e-9
    assert abs(r2["final_cost"] - g2.stats["final_cost"]) / g2.stats["final_cost"] < 1e-9


def test_fp64_solve_is_bitwise_repeatable(ctx):
    p = Synth(2, n_windows=1, seed=9).window(0)
    o = workload_options(2)
    a, b = ctx.solve(p, o), ctx.solve(p, o)
    assert np.array_equal(a.points, b.points) and np.array_equal(a.cost_trace, b.cost_trace)
