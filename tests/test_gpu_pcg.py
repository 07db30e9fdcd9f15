"""GPU parity of the PCG solver and the shared radial distortion (the large robust workload's
solver, family 4) against the CPU oracle running the same algorithm (block-Jacobi PCG on the
reduced system, convergence tested every 4 iterations).

FP64: final cost within 1e-6 relative of the oracle.  Mixed precision (FP32 Jacobians and
reduced-camera products): the robust problem is still descending ~1e-4 per iteration after 15
iterations, so FP32 rounding of the steps moves the end point along the descent; the bar is that
mixed ends no more than 1e-6 above the FP64 oracle's cost (the same final cost or better) and
within 1e-5 of it either way."""
import numpy as np
import pytest

from nav24_gb300 import abi
from nav24_gb300.synth import Synth, workload_options
from oracle import oracle

pytestmark = pytest.mark.gpu


def rel(a, b):
    return abs(a - b) / abs(b)


def test_pcg_without_distortion_matches_oracle(ctx):
    p = Synth(1, n_cams=40, n_points=3000, seed=5).window(0)
    o = abi.default_options(iterations=10, robust=1, huber_delta=2.0, solver=abi.SOLVER_PCG,
                            pcg_tolerance=1e-10, pcg_max_iterations=400)
    g = ctx.solve(p, o)
    r = oracle.solve(p, o, n_threads=8)
    assert g.status == abi.OK and g.stats["pcg_iterations_total"] > 0
    assert rel(g.stats["final_cost"], r.stats["final_cost"]) < 1e-6


@pytest.mark.parametrize("precision", [abi.FP64, abi.MIXED])
def test_pcg_with_distortion_matches_oracle(ctx, precision):
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
