"""The large robust workload at full size against the FP64 oracle: 1000 cameras along a 2,000 m
figure-eight (three loops), 500,000 points, ~4M observations, shared radial k1, k2 optimized, 5%
outliers, Huber 1.5 px, block-Jacobi PCG (tolerance 1e-6, at most 100 iterations), 30 LM iterations
(family 4, seed 1004).  The oracle runs the same algorithm (block-sparse reduced system) on every
host core.  Both GPU forms end within 1e-6 relative of the oracle's final cost, and the FP64 form's
recovered distortion agrees with the oracle's."""
import os

import numpy as np
import pytest

from nav24_gb300 import abi
from nav24_gb300.synth import Synth, workload_options
from oracle import oracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def eight():
    p = Synth(4).window(0)
    assert p.n_cams == 1000 and p.n_points == 500000 and p.n_obs > 3_900_000
    r = oracle.solve(p, workload_options(4), n_threads=max(1, os.cpu_count() or 1))
    assert r.status == abi.OK
    return p, r


@pytest.mark.parametrize("precision", [abi.FP64, abi.MIXED])
def test_figure_eight_full_size_matches_oracle(ctx, eight, precision):
    p, r = eight
    g = ctx.solve(p, workload_options(4, precision=precision))
    assert g.status == abi.OK and g.stats["iterations_done"] == 30
    rel = abs(g.stats["final_cost"] - r.stats["final_cost"]) / r.stats["final_cost"]
    assert rel < 1e-6, rel
    if precision == abi.FP64:
        assert np.max(np.abs(g.intrinsics[4:6] - r.intrinsics[4:6])) < 1e-6
