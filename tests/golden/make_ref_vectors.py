"""Generate tests/golden/ref_edges.npz: residuals, Jacobians and depth tests computed by nav24's own
code, compiled from the reference tree by oracle/ref_build.py (EdgeSE3ProjectXYZ::computeError,
isDepthPositive and linearizeOplus, core/dataTypes/optimization/OptimizableTypes.hpp:102-113 and
OptimizableTypes.cpp:140-161, through Calibration::project/projectJac, core/sensor/camera/
Calibration.cpp:235-247, into Pinhole.cpp:30-36,70-80 and KannalaBrandt8.cpp:80-107,195-226).

    python tests/golden/make_ref_vectors.py

The problems are the cases of tests/ref_cases.py; for each, N_SAMPLE evenly spaced observations
are kept: their index, e [2], jc [2][6] (pose, rotation first), jp [2][3] (point) and the depth
test.  The GPU host has no reference tree, so its tests read this file.
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(HERE.parent))

from oracle import ref  # noqa: E402
from ref_cases import CASES, sample  # noqa: E402


def main() -> None:
    if ref.lib() is None:
        raise SystemExit("the reference tree is needed to build oracle/_ref")
    out = {}
    for name, make in CASES.items():
        p = make()
        e, jc, jp, dpos = ref.edges(p)
        idx = sample(p.n_obs)
        out[f"{name}/idx"] = idx
        out[f"{name}/n_obs"] = np.int64(p.n_obs)
        out[f"{name}/e"] = e[idx]
        out[f"{name}/jc"] = jc[idx]
        out[f"{name}/jp"] = jp[idx]
        out[f"{name}/depth_positive"] = dpos[idx]
        print(f"{name}: {p.n_obs} observations, {idx.size} kept, {int((dpos == 0).sum())} with depth <= 0")
    np.savez_compressed(HERE / "ref_edges.npz", **out)


if __name__ == "__main__":
    main()
