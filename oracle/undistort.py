"""CPU restatement of keypoint undistortion (test infrastructure only).

nav24: Calibration::undistort (core/sensor/camera/Calibration.cpp:135-148) -> PinholeRadTan::
UndistortKeyPoints (core/sensor/camera/models/PinholeRadTan.cpp:11-24) -> cv::undistortPoints with
R = I, P = K and distortion (k1, k2, p1, p2).  OpenCV (>= 4.2.0, not present here) inverts the
distortion by the fixed-point iteration below on normalized coordinates, 5 times by default.
"""
from __future__ import annotations

import numpy as np


def undistort(K, dist, uv, iterations=5):
    fx, fy, cx, cy = K
    k1, k2, p1, p2 = dist
    x0 = (uv[:, 0] - cx) / fx
    y0 = (uv[:, 1] - cy) / fy
    x, y = x0.copy(), y0.copy()
    for _ in range(iterations):
        r2 = x * x + y * y
        icd = 1.0 / (1.0 + (k2 * r2 + k1) * r2)
        dx = 2.0 * p1 * x * y + p2 * (r2 + 2.0 * x * x)
        dy = p1 * (r2 + 2.0 * y * y) + 2.0 * p2 * x * y
        x = (x0 - dx) * icd
        y = (y0 - dy) * icd
    return np.stack([fx * x + cx, fy * y + cy], axis=1)


def distort(K, dist, uv):
    """The forward model (the distortion the iteration inverts), for round-trip checks."""
    fx, fy, cx, cy = K
    k1, k2, p1, p2 = dist
    x = (uv[:, 0] - cx) / fx
    y = (uv[:, 1] - cy) / fy
    r2 = x * x + y * y
    rad = 1.0 + k1 * r2 + k2 * r2 * r2
    xd = x * rad + 2.0 * p1 * x * y + p2 * (r2 + 2.0 * x * x)
    yd = y * rad + p1 * (r2 + 2.0 * y * y) + 2.0 * p2 * x * y
    return np.stack([fx * xd + cx, fy * yd + cy], axis=1)
