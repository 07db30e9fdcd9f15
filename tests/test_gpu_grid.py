"""GPU parity tests of the grid engine (one large problem on the whole GPU: more than 24 free
cameras) against the CPU oracle, with the same tolerances as the window engine: reduced-system
pattern bit-exact and values within 1e-10 relative (FP64), final cost within 1e-6 relative after
a fixed number of LM iterations, and the mixed form within 1e-6 of the FP64 oracle."""
import numpy as np
import pytest

from nav24_gb300 import abi
from nav24_gb300.synth import Synth, workload_options
from oracle import oracle

pytestmark = pytest.mark.gpu


def rel(a, b):
    return abs(a - b) / abs(b)


def grid_problem():
    return Synth(1, n_cams=50, n_points=4000, seed=77).window(0)  # 49 free cameras


def test_grid_reduced_system_matches_oracle(ctx):
    p = grid_problem()
    o = abi.default_options(robust=1, huber_delta=2.0)
    gS, gb, gidx = ctx.reduced_system(p, o, 1e-2)
    oS, ob, oidx = oracle.reduced_system(p, o, 1e-2)
    assert np.array_equal(gidx, oidx)
    nf = oS.shape[0] // 6
    blk = lambda S: np.array([[np.any(S[6 * a:6 * a + 6, 6 * b:6 * b + 6] != 0) for b in range(nf)] for a in range(nf)])
    assert np.array_equal(blk(gS), blk(oS))
    assert np.max(np.abs(gS - oS)) / np.max(np.abs(oS)) < 1e-10
    assert np.max(np.abs(gb - ob)) / np.max(np.abs(ob)) < 1e-10


@pytest.mark.parametrize("robust", [0, 1])
def test_grid_fp64_solve_matches_oracle(ctx, robust):
    p = grid_problem()
    o = abi.default_options(iterations=10, robust=robust, huber_delta=2.0)
    g = ctx.solve(p, o)
    r = oracle.solve(p, o, n_threads=8)
    assert g.status == abi.OK and g.stats["n_free_cams"] == 49
    assert rel(g.stats["initial_cost"], r.stats["initial_cost"]) < 1e-12
    assert rel(g.stats["final_cost"], r.stats["final_cost"]) < 1e-6
    n = min(len(g.cost_trace), len(r.cost_trace))
    assert np.max(np.abs(g.cost_trace[:n] - r.cost_trace[:n]) / r.cost_trace[:n]) < 1e-6
    assert np.allclose(g.points, r.points, rtol=0, atol=1e-6)


def test_grid_mixed_reaches_fp64_cost(ctx):
    p = grid_problem()
    o = abi.default_options(iterations=20, robust=1, huber_delta=2.0)
    r = oracle.solve(p, o, n_threads=8)
    o.precision = abi.MIXED
    g = ctx.solve(p, o)
    assert rel(g.stats["final_cost"], r.stats["final_cost"]) < 1e-6


def test_cap_workload_fp64(ctx):
    p = Synth(3, n_points=3000).window(0)  # 50 cameras on a sphere cap, dense reduced system
    o = workload_options(3)
    g = ctx.solve(p, o)
    r = oracle.solve(p, o, n_threads=8)
    assert rel(g.stats["final_cost"], r.stats["final_cost"]) < 1e-6


def test_grid_workload_full_size(ctx):
    """The 200-camera grid workload (family 1): FP64 and mixed forms against the FP64 oracle."""
    p = Synth(1).window(0)
    o = workload_options(1)
    r = oracle.solve(p, o, n_threads=16)
    g = ctx.solve(p, o)
    assert rel(g.stats["final_cost"], r.stats["final_cost"]) < 1e-6
    g = ctx.solve(p, workload_options(1, abi.MIXED))
    assert rel(g.stats["final_cost"], r.stats["final_cost"]) < 1e-6


@pytest.mark.parametrize("solver", [abi.SOLVER_CHOLESKY, abi.SOLVER_PCG])
def test_grid_host_structure_passes_agree(ctx, monkeypatch, solver):
    """The reduced system's pair lists are built point-major with a dense block map up to 4096 free
    cameras and per camera row beyond; both give the same lists, so the solves agree bit for bit
    (NAVBA_GRID_HOST=rows forces the per-row passes)."""
    p = Synth(4, n_cams=60, n_points=6000, seed=8).window(0)
    o = workload_options(4)
    o.iterations = 6
    o.solver = solver
    o.optimize_distortion = 1 if solver == abi.SOLVER_PCG else 0
    res = []
    for mode in ("", "rows"):
        monkeypatch.setenv("NAVBA_GRID_HOST", mode)
        res.append(ctx.solve(p, o))
    a, b = res
    assert a.status == abi.OK and b.status == abi.OK
    assert np.array_equal(a.cam_pose, b.cam_pose) and np.array_equal(a.points, b.points)
    assert np.array_equal(a.cost_trace, b.cost_trace, equal_nan=True)


@pytest.mark.parametrize("precision", [abi.FP64, abi.MIXED])
def test_grid_solve_forms_agree(ctx, monkeypatch, precision):
    """The triangular solves keep x in shared memory when it fits and in global memory beyond
    (NAVBA_SOLVE_GLOBAL_X=1 forces the latter); both run the same operations in the same order, so
    the solves agree bit for bit."""
    p = grid_problem()
    o = abi.default_options(iterations=6, robust=1, huber_delta=2.0)
    o.precision = precision
    res = []
    for mode in ("", "1"):
        monkeypatch.setenv("NAVBA_SOLVE_GLOBAL_X", mode)
        res.append(ctx.solve(p, o))
    a, b = res
    assert a.status == abi.OK and b.status == abi.OK
    assert np.array_equal(a.cam_pose, b.cam_pose) and np.array_equal(a.points, b.points)
    assert np.array_equal(a.cost_trace, b.cost_trace, equal_nan=True)


@pytest.mark.parametrize("precision", [abi.FP64, abi.MIXED])
@pytest.mark.parametrize("solver", [abi.SOLVER_CHOLESKY, abi.SOLVER_PCG])
def test_grid_workspace_reuse(product_lib, monkeypatch, solver, precision):
    """A context keeps its grid solves' device buffers (one slab, grown at the end of a call to
    what the call needed) and pinned read-back memory.  Solves of a small and a larger problem,
    alternated on one context (the slab too small, then large enough, then reused), match the
    same solves on contexts that allocate per call (NAVBA_GRID_WORKSPACE=0) bit for bit."""
    from nav24_gb300 import Context

    small = grid_problem()
    large = Synth(4, n_cams=60, n_points=6000, seed=8).window(0)
    o = workload_options(4, precision)
    o.iterations = 4
    o.solver = solver
    o.optimize_distortion = 1 if solver == abi.SOLVER_PCG else 0
    seq = [small, large, small, large]
    with Context(0) as c:
        kept = [c.solve(p, o) for p in seq]
    monkeypatch.setenv("NAVBA_GRID_WORKSPACE", "0")
    with Context(0) as c:
        fresh = [c.solve(p, o) for p in seq]
    for a, b in zip(kept, fresh):
        assert a.status == abi.OK and b.status == abi.OK
        assert np.array_equal(a.cam_pose, b.cam_pose) and np.array_equal(a.points, b.points)
        assert np.array_equal(a.cost_trace, b.cost_trace, equal_nan=True)
