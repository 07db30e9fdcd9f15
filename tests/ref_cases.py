"""Problems on which nav24's own edge code (built in oracle/_ref from the reference tree) was
evaluated to make tests/golden/ref_edges.npz.  Each case regenerates the same problem on any host:
the synthetic families are host-independent (their digests are pinned in synth_digests.json) and the
rest is seeded numpy arithmetic of exactly representable values.

Every case's intrinsics are float values, as nav24 keeps them (Calibration.cpp:42-60 rounds each
parameter to float), so the double inputs of the oracle and the GPU equal the reference's."""
from __future__ import annotations

import numpy as np

from nav24_gb300 import abi
from nav24_gb300.synth import Synth

from kb8_util import kb8_problem

N_SAMPLE = 500  # edges kept per case in the fixture


def _f32(p: abi.Problem) -> abi.Problem:
    p.intrinsics = p.intrinsics.astype(np.float32).astype(np.float64)
    return p


def _behind() -> abi.Problem:
    """200 observations of points around 8 cameras at depths in [-3, 3] m (|z| >= 0.05): the depth
    test (isDepthPositive) sees both signs."""
    rng = np.random.default_rng(77)
    nc, npt = 8, 100
    poses = np.zeros((nc, 12))
    for c in range(nc):
        a = 0.3 * c
        R = np.array([[np.cos(a), 0, np.sin(a)], [0, 1, 0], [-np.sin(a), 0, np.cos(a)]])
        P = np.zeros((3, 4))
        P[:, :3] = R
        P[:, 3] = rng.uniform(-0.5, 0.5, 3)
        poses[c] = P.reshape(-1)
    pts = rng.uniform(-2.0, 2.0, (npt, 3))
    obs_cam = rng.integers(0, nc, 200).astype(np.int32)
    obs_pt = rng.integers(0, npt, 200).astype(np.int32)
    P = poses.reshape(-1, 3, 4)
    z = np.einsum("ij,ij->i", P[obs_cam, 2, :3], pts[obs_pt]) + P[obs_cam, 2, 3]
    keep = np.abs(z) >= 0.05
    obs_cam, obs_pt = obs_cam[keep], obs_pt[keep]
    uv = rng.uniform(0.0, 640.0, (obs_cam.size, 2))
    return abi.Problem(cam_pose=poses, points=pts, obs_uv=uv, obs_cam=obs_cam, obs_point=obs_pt,
                       intrinsics=np.array([500.0, 500.0, 320.0, 240.0, 0, 0, 0, 0]))


def _pinhole(p: abi.Problem) -> abi.Problem:
    p.camera_model = abi.CAM_PINHOLE
    p.intrinsics[4:] = 0.0
    return p


CASES = {
    # the plain small workload (10 cameras on a ring, 500 points)
    "ring": lambda: _f32(Synth(0).window(0)),
    # one window of the batched family
    "window": lambda: _f32(Synth(2, n_windows=2).window(1)),
    # a piece of the figure-eight (large world coordinates), pinhole
    "eight": lambda: _f32(_pinhole(Synth(4, n_cams=20, n_points=2000).window(0))),
    # the Kannala-Brandt 8 model
    "kb8": lambda: _f32(kb8_problem(n_cams=12, n_points=500)),
    # points on both sides of the cameras
    "behind": lambda: _f32(_behind()),
}


def sample(n_obs: int) -> np.ndarray:
    """The edges kept in the fixture: N_SAMPLE evenly spaced observation indices (all if fewer)."""
    if n_obs <= N_SAMPLE:
        return np.arange(n_obs, dtype=np.int32)
    return np.linspace(0, n_obs - 1, N_SAMPLE).round().astype(np.int32)
