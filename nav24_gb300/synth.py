"""Seeded synthetic BA workloads (wraps libnavsynth.so, include/nav_ba_synth.h).

Workload families and the seeds of the five named workloads (seed = 1000 + family):
  0 ring    10 cams, 500 points, camera 0 fixed, 10 LM iterations, lambda0 = 1e-3
  1 grid    200 cams on a 20 x 10 grid facing down, 50,000 points, Huber 2 px, 20 iterations
  2 windows 512 local windows, 5-20 keyframes, 200-3000 points, first two keyframes fixed
  3 cap     50 cams on a sphere cap, 10,000 points, about 6 views per point
  4 eight   1000 cams on a figure-eight, 500,000 points, radial k1/k2, 5% outliers, Huber 1.5 px
"""
from __future__ import annotations

import ctypes as C
import hashlib
from pathlib import Path

import numpy as np

from . import abi

_LIB = None


def _lib():
    global _LIB
    if _LIB is None:
        from .build import build_synth
        path = build_synth()  # rebuilds only when a source or header is newer than the library
        lib = C.CDLL(str(path))
        lib.nav_synth_create.restype = C.c_void_p
        lib.nav_synth_create.argtypes = [C.POINTER(abi.nav_synth_params)]
        lib.nav_synth_destroy.argtypes = [C.c_void_p]
        lib.nav_synth_counts.argtypes = [C.c_void_p] + [C.POINTER(C.c_int64)] * 4 + [C.POINTER(C.c_int32)]
        lib.nav_synth_size.restype = C.c_int64
        lib.nav_synth_size.argtypes = [C.c_void_p, C.c_int32]
        lib.nav_synth_copy.restype = C.c_int32
        lib.nav_synth_copy.argtypes = [C.c_void_p, C.c_int32, C.c_void_p]
        _LIB = lib
    return _LIB


_DT = {0: np.float64, 1: np.float64, 2: np.uint8, 3: np.float64, 4: np.float64, 5: np.uint8,
       6: np.float64, 7: np.int32, 8: np.int32, 9: np.int64, 10: np.int64, 11: np.int64,
       12: np.float64, 13: np.float64}


class Synth:
    """One generated workload: all arrays as numpy, windows as Problem views."""

    def __init__(self, family: int, seed: int | None = None, n_cams: int = 0, n_points: int = 0,
                 n_windows: int = 0, pixel_noise: float = -1.0, outlier_frac: float = -1.0,
                 rot_perturb: float = -1.0, trans_perturb: float = -1.0,
                 point_perturb: float = -1.0, min_cams: int = 0, min_points: int = 0):
        lib = _lib()
        p = abi.nav_synth_params()
        p.family = family
        p.n_cams = n_cams
        p.n_points = n_points
        p.n_windows = n_windows
        p.seed = 1000 + family if seed is None else seed
        p.pixel_noise = pixel_noise
        p.outlier_frac = outlier_frac
        p.rot_perturb = rot_perturb
        p.trans_perturb = trans_perturb
        p.point_perturb = point_perturb
        p.min_cams = min_cams
        p.min_points = min_points
        h = lib.nav_synth_create(C.byref(p))
        if not h:
            raise ValueError("invalid synth parameters")
        try:
            nw, nc, npt, no = (C.c_int64(), C.c_int64(), C.c_int64(), C.c_int64())
            model = C.c_int32()
            lib.nav_synth_counts(h, C.byref(nw), C.byref(nc), C.byref(npt), C.byref(no), C.byref(model))
            arrs = {}
            for aid, dt in _DT.items():
                n = lib.nav_synth_size(h, aid)
                a = np.zeros(max(n, 0), dt)
                if n > 0:
                    lib.nav_synth_copy(h, aid, a.ctypes.data)
                arrs[aid] = a
        finally:
            lib.nav_synth_destroy(h)
        self.family = family
        self.seed = p.seed
        self.camera_model = model.value
        self.cam_pose = arrs[0].reshape(-1, 12)
        self.cam_pose_true = arrs[1].reshape(-1, 12)
        self.cam_fixed = arrs[2]
        self.points = arrs[3].reshape(-1, 3)
        self.points_true = arrs[4].reshape(-1, 3)
        self.point_fixed = arrs[5]
        self.obs_uv = arrs[6].reshape(-1, 2)
        self.obs_cam = arrs[7]
        self.obs_point = arrs[8]
        self.win_cam = arrs[9]
        self.win_pt = arrs[10]
        self.win_obs = arrs[11]
        self.intrinsics = arrs[12]
        self.intrinsics_init = arrs[13]

    def digest(self) -> str:
        """SHA-256 of every generated array: the generator is host-independent (no platform libm,
        no floating-point contraction), so a workload has the same digest on every machine."""
        h = hashlib.sha256()
        for a in (self.cam_pose, self.cam_pose_true, self.cam_fixed, self.points, self.points_true,
                  self.point_fixed, self.obs_uv, self.obs_cam, self.obs_point, self.win_cam, self.win_pt,
                  self.win_obs, self.intrinsics, self.intrinsics_init):
            h.update(np.ascontiguousarray(a).tobytes())
        return h.hexdigest()

    @property
    def n_windows(self) -> int:
        return len(self.win_cam) - 1

    @property
    def n_obs(self) -> int:
        return self.obs_uv.shape[0]

    def window(self, w: int = 0, truth: bool = False) -> abi.Problem:
        c0, c1 = self.win_cam[w], self.win_cam[w + 1]
        p0, p1 = self.win_pt[w], self.win_pt[w + 1]
        o0, o1 = self.win_obs[w], self.win_obs[w + 1]
        return abi.Problem(
            cam_pose=(self.cam_pose_true if truth else self.cam_pose)[c0:c1],
            points=(self.points_true if truth else self.points)[p0:p1],
            obs_uv=self.obs_uv[o0:o1], obs_cam=self.obs_cam[o0:o1], obs_point=self.obs_point[o0:o1],
            intrinsics=self.intrinsics if truth else self.intrinsics_init,
            cam_fixed=self.cam_fixed[c0:c1], point_fixed=self.point_fixed[p0:p1],
            camera_model=self.camera_model)

    def windows(self) -> list[abi.Problem]:
        return [self.window(w) for w in range(self.n_windows)]

    def pose_problems(self) -> list[abi.PoseProblem]:
        """Tracking problems: per window, its last camera (perturbed initial pose) against the window's
        points seen by it, held fixed at their initial positions (the current frame optimized against
        a fixed map, as in FE_SlamMonoV.cpp:153-165)."""
        out = []
        for w in range(self.n_windows):
            c0, c1 = self.win_cam[w], self.win_cam[w + 1]
            p0 = self.win_pt[w]
            o0, o1 = self.win_obs[w], self.win_obs[w + 1]
            cam = c1 - c0 - 1
            sel = np.nonzero(self.obs_cam[o0:o1] == cam)[0] + o0
            out.append(abi.PoseProblem(pose=self.cam_pose[c1 - 1], points=self.points[p0 + self.obs_point[sel]],
                                       obs_uv=self.obs_uv[sel], intrinsics=self.intrinsics_init,
                                       camera_model=self.camera_model))
        return out


# Named workloads (one per family) with their solver options.
def workload_options(family: int, precision: int = abi.FP64) -> abi.nav_ba_options:
    if family == 0:
        return abi.default_options(iterations=10, initial_lambda=1e-3, precision=precision)
    if family == 1:
        return abi.default_options(iterations=20, robust=1, huber_delta=2.0, precision=precision)
    if family == 2:
        return abi.default_options(iterations=10, precision=precision)
    if family == 3:
        return abi.default_options(iterations=5, robust=1, huber_delta=2.0, precision=precision)
    if family == 4:
        return abi.default_options(iterations=30, robust=1, huber_delta=1.5, precision=precision,
                                   solver=abi.SOLVER_PCG, optimize_distortion=1,
                                   pcg_tolerance=1e-6, pcg_max_iterations=100)
    raise ValueError(family)
