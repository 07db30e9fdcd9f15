"""GPU test of nav_ba_solve_noalloc, the entry point for callers that must not allocate device
memory while solving (a real-time tracking thread, or a process whose device memory belongs to
another framework's allocator).  It solves one window in the library's static device array.

The test calls it through the C ABI twice in a row (the second call reuses the array the first one
left behind) and compares both results with nav_ba_solve on the same problem, within the parity
tolerances used for the FP64 and mixed forms.  A second test checks the property the entry point
exists for: after a first call, further calls leave the device's free memory unchanged, while
nav_ba_solve on a new context, the control, takes device memory for its buffers.  This file is
collected last on purpose."""
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
                # the same transfer and timing statistics as nav_ba_solve reports
                assert got.stats["h2d_bytes"] > 0 and got.stats["d2h_bytes"] > 0, (name, call)
                assert got.stats["time_solve_ms"] > 0.0, (name, call)


def test_noalloc_leaves_device_memory_unchanged():
    torch = pytest.importorskip("torch")
    prob = Synth(2, n_windows=1, seed=31).window(0)
    opt = abi.default_options(iterations=10, robust=1, huber_delta=2.0)
    with Context(0) as ctx:
        for precision in (abi.FP64, abi.MIXED):  # first calls: lazy module loading, the arena address
            opt.precision = precision
            ctx.solve_noalloc(prob, opt)
        torch.cuda.synchronize(0)
        free0 = torch.cuda.mem_get_info(0)[0]
        for _ in range(3):
            for precision in (abi.FP64, abi.MIXED):
                opt.precision = precision
                assert ctx.solve_noalloc(prob, opt).status == abi.OK
        assert torch.cuda.mem_get_info(0)[0] == free0
        # control: nav_ba_solve of a 64-window batch on a fresh context allocates its device buffers
        with Context(0) as ctx2:
            batch = Synth(2, n_windows=64, seed=32).windows()
            opt.precision = abi.MIXED
            ctx2.solve_batched(batch, opt)
            assert torch.cuda.mem_get_info(0)[0] < free0


def test_noalloc_rejects_problems_beyond_its_limits():
    with Context(0) as ctx:
        big = Synth(3, n_cams=12, n_points=5000).window(0)  # more than NAV_BA_NOALLOC_MAX_POINTS
        r = ctx.solve_noalloc(big, workload_options(3), raise_on_error=False)
        assert r.status == abi.ERR_UNSUPPORTED
        assert "no-allocation limits" in ctx.last_error()
        assert not np.any(r.points)
