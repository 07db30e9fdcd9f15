"""CPU restatement of TwoViewReconstruction::Triangulate and CheckRT (test infrastructure only).

Follows core/operators/mapInit/OP_2ViewReconstruction.cpp: Triangulate (:1179-1193) builds the 4x4
DLT matrix from P1 = K[I|0] and P2 = K[R|t] and takes the last row of V^T of its SVD (numpy's LAPACK
SVD in FP64 where the reference runs cv::SVD on CV_32F); CheckRT (:1244-1353) checks every inlier
match in order - finite point, depth in front of camera 1 and camera 2 unless the parallax is small,
squared reprojection error in both images - counts the passing ones (nGood), marks those with enough
parallax (vbGood), and reports acos of the sorted cos-parallax at index min(minTriangulated, n-1).
"""
from __future__ import annotations

import numpy as np


def triangulate(K, kp1, kp2, R, t):
    fx, fy, cx, cy = K
    Km = np.array([[fx, 0, cx], [0, fy, cy], [0, 0, 1.0]])
    P1 = np.hstack([Km, np.zeros((3, 1))])
    P2 = Km @ np.hstack([R, t.reshape(3, 1)])
    A = np.stack([kp1[0] * P1[2] - P1[0], kp1[1] * P1[2] - P1[1], kp2[0] * P2[2] - P2[0], kp2[1] * P2[2] - P2[1]])
    _, _, vt = np.linalg.svd(A)
    x = vt[3]
    return x[:3] / x[3]


def check_rt(K, kp1, kp2, R, t, th2, min_parallax_cos, min_triangulated, inlier=None, quantities=None):
    """quantities: a dict that receives, per match, the values CheckRT compares with its thresholds
    (z1, z2: depths in the two cameras, r1, r2: the point's distances from them; err1, err2: squared
    reprojection errors; cos: cos-parallax); NaN where a match has no finite point."""
    fx, fy, cx, cy = K
    n = kp1.shape[0]
    pts = np.full((n, 3), np.nan)
    tri = np.zeros(n, bool)
    good = np.zeros(n, bool)
    cosp = np.full(n, np.nan)
    qv = {k: np.full(n, np.nan) for k in ("z1", "z2", "r1", "r2", "err1", "err2", "cos")}
    O2 = -R.T @ t
    for i in range(n):
        if inlier is not None and not inlier[i]:
            continue
        with np.errstate(all="ignore"):
            p = triangulate(K, kp1[i], kp2[i], R, t)
        if not np.all(np.isfinite(p)):
            continue
        pts[i] = p
        n2 = p - O2
        c = p @ n2 / (np.linalg.norm(p) * np.linalg.norm(n2))
        cosp[i] = c
        q = R @ p + t
        e1 = (fx * p[0] / p[2] + cx - kp1[i, 0]) ** 2 + (fy * p[1] / p[2] + cy - kp1[i, 1]) ** 2
        e2 = (fx * q[0] / q[2] + cx - kp2[i, 0]) ** 2 + (fy * q[1] / q[2] + cy - kp2[i, 1]) ** 2
        qv["z1"][i], qv["z2"][i], qv["err1"][i], qv["err2"][i], qv["cos"][i] = p[2], q[2], e1, e2, c
        qv["r1"][i], qv["r2"][i] = np.linalg.norm(p), np.linalg.norm(q)
        if p[2] <= 0 and c < min_parallax_cos:
            continue
        if q[2] <= 0 and c < min_parallax_cos:
            continue
        if e1 > th2:
            continue
        if e2 > th2:
            continue
        tri[i] = True
        good[i] = c < min_parallax_cos
    if quantities is not None:
        quantities.update(qv)
    cs = np.sort(cosp[tri])
    par = float(np.degrees(np.arccos(cs[min(min_triangulated, len(cs) - 1)]))) if len(cs) else 0.0
    return pts, tri, good, int(tri.sum()), par
