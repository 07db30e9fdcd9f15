"""GPU test of nav_ba_solve_noalloc, the entry point for callers that must not allocate device
memory while solving (a real-time tracking thread, or a process whose device memory belongs to
another framework's allocator).  It solves one window in the library's static device array.

The test calls it through the C ABI twice in a row (the second call reuses the array the first one
left behind) and compares both results with nav_ba_solve on the same problem, within the parity
tolerances used for the FP64 and mixed forms.  This file is collected last on purpose."""
import numpy as np
import pytest

from nav24_gb300 import Context, abi
from nav24_gb300.synth import Synth, workload_options

pytestmark = pytest.mark.gpu


def _problems():
    return [
        ("ring", Synth(0).window(0), workload_options(0)),
        ("window", Synth(2, n_windows=1, seed=31).window(0), abi.default_options(iterations=10, robust=1,
                                                                                  huber_delta=2.0)),
    ]


@pytest.mark.parametrize("precision", [abi.FP64, abi.MIXED])
def test_noalloc_matches_solve_on_two_calls(precision):
    with Context(0) as ctx:
        for name, prob, opt in _problems():
            opt.precision = precision
            ref = ctx.solve(prob, opt)
            assert ref.status == abi.OK, name
            rtol = 1e-9 if precision == abi.FP64 else 1e-6
            for call in range(2):
                got = ctx.solve_noalloc(prob, opt)
                assert got.status == abi.OK, (name, call)
                rel = abs(got.stats["final_cost"] - ref.stats["final_cost"]) / ref.stats["final_cost"]
                assert rel < rtol, (name, call, rel)
                assert abs(got.stats["initial_cost"] - ref.stats["initial_cost"]) / ref.stats["initial_cost"] < 1e-12
                assert np.allclose(got.points, ref.points, rtol=0, atol=1e-5), (name, call)
                assert np.allclose(got.cam_pose, ref.cam_pose, rtol=0, atol=1e-6), (name, call)
                assert got.stats["n_active_edges"] == ref.stats["n_active_edges"]


def test_noalloc_rejects_problems_beyond_its_limits():
    with Context(0) as ctx:
        big = Synth(3, n_cams=12, n_points=5000).window(0)  # more than NAV_BA_NOALLOC_MAX_POINTS
        r = ctx.solve_noalloc(big, workload_options(3), raise_on_error=False)
        assert r.status == abi.ERR_UNSUPPORTED
        assert "no-allocation limits" in ctx.last_error()
        assert not np.any(r.points)
