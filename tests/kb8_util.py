"""Kannala-Brandt test problems (numpy): the synthetic geometry observed through the fisheye model
of core/sensor/camera/models/KannalaBrandt8.cpp:80-107 (theta = atan2(rho, z), r(theta) =
theta + k1 theta^3 + k2 theta^5 + k3 theta^7 + k4 theta^9, pi = f r (cos psi, sin psi) + c)."""
import numpy as np

from nav24_gb300 import abi
from nav24_gb300.synth import Synth

KB8 = np.array([380.0, 380.0, 320.0, 240.0, -0.012, 0.0025, -0.0006, 0.00008])


def kb8_project(k, Xc, float_angles=False):
    """The reference's projection; float_angles=True rounds theta and psi through float32 as its
    project does (atan2f, sqrtf)."""
    x, y, z = Xc[:, 0], Xc[:, 1], Xc[:, 2]
    if float_angles:
        f32 = np.float32
        th = np.arctan2(np.sqrt(f32(x * x + y * y)), f32(z)).astype(np.float64)
        psi = np.arctan2(f32(y), f32(x)).astype(np.float64)
    else:
        th = np.arctan2(np.sqrt(x * x + y * y), z)
        psi = np.arctan2(y, x)
    r = th + k[4] * th ** 3 + k[5] * th ** 5 + k[6] * th ** 7 + k[7] * th ** 9
    return np.stack([k[0] * r * np.cos(psi) + k[2], k[1] * r * np.sin(psi) + k[3]], axis=1)


def transform(p: abi.Problem):
    P = p.cam_pose.reshape(-1, 3, 4)
    R, t = P[:, :, :3], P[:, :, 3]
    return np.einsum("nij,nj->ni", R[p.obs_cam], p.points[p.obs_point]) + t[p.obs_cam]


def kb8_problem(family=3, seed=5, noise=0.7, **kw):
    s = Synth(family, seed=seed, **kw)
    truth, init = s.window(0, truth=True), s.window(0)
    rng = np.random.default_rng(seed)
    uv = kb8_project(KB8, transform(truth)) + noise * rng.standard_normal((truth.n_obs, 2))
    q = init.copy()
    q.obs_uv = np.ascontiguousarray(uv)
    q.intrinsics = KB8.copy()
    q.camera_model = abi.CAM_KANNALA_BRANDT8
    return q
