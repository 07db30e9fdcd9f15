"""Seeded two-view matches for the triangulation tests: camera 1 at the origin, camera 2 at
(R, t) with a 0.3 m baseline, points 2-8 m ahead, 0.5 px noise, 10% outlier matches (random
pixels), and the four relative poses of an essential-matrix decomposition (R or the twisted
R' = rot(t, pi) R, with +t or -t)."""
import numpy as np
from scipy.spatial.transform import Rotation

K = np.array([500.0, 500.0, 320.0, 240.0])


def project(P):
    return np.stack([K[0] * P[:, 0] / P[:, 2] + K[2], K[1] * P[:, 1] / P[:, 2] + K[3]], axis=1)


def scene(n=2000, seed=3):
    rng = np.random.default_rng(seed)
    R = Rotation.from_rotvec([0.02, -0.06, 0.01]).as_matrix()
    t = np.array([-0.3, 0.02, 0.01])
    X = np.stack([rng.uniform(-2, 2, n), rng.uniform(-1.5, 1.5, n), rng.uniform(2, 8, n)], axis=1)
    kp1 = project(X) + 0.5 * rng.standard_normal((n, 2))
    kp2 = project(X @ R.T + t) + 0.5 * rng.standard_normal((n, 2))
    out = rng.random(n) < 0.1
    kp2[out] = np.stack([rng.uniform(0, 640, out.sum()), rng.uniform(0, 480, out.sum())], axis=1)
    inlier = rng.random(n) > 0.05
    tw = Rotation.from_rotvec(np.pi * t / np.linalg.norm(t)).as_matrix()
    Rs = np.stack([R, R, tw @ R, tw @ R])
    ts = np.stack([t, -t, t, -t])
    return kp1, kp2, inlier, Rs, ts, X
