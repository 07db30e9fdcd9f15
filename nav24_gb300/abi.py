"""ctypes mirror of include/nav_ba.h and include/nav_ba_synth.h, plus numpy marshalling.

The struct layouts here must match the C headers field for field; ``tests/test_abi.py`` checks
the sizes against the compiled libraries.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

# --- status codes and enums (include/nav_ba.h) ----------------------------------------------
OK = 0
EMPTY = 1
ERR_ARGUMENT = -1
ERR_NONFINITE_INPUT = -2
ERR_NONFINITE_COST = -3
ERR_CUDA = -4
ERR_OUT_OF_MEMORY = -5
ERR_UNSUPPORTED = -6
ERR_DEVICE_TIMEOUT = -7
ERR_NO_DEVICE = -8

CAM_PINHOLE = 0
CAM_PINHOLE_RADIAL = 1
CAM_KANNALA_BRANDT8 = 2
FP64 = 0
MIXED = 1
SOLVER_CHOLESKY = 0
SOLVER_PCG = 1

TERM_ITERATIONS = 0
TERM_TRIALS_EXHAUSTED = 1
TERM_ZERO_GAIN = 2
TERM_LAMBDA_NONFINITE = 3
TERM_NOTHING_TO_DO = 4

WINDOW_MAX_CAMS = 24

_dp = C.POINTER(C.c_double)
_u8p = C.POINTER(C.c_uint8)
_i32p = C.POINTER(C.c_int32)


class nav_ba_problem(C.Structure):
    _fields_ = [
        ("n_cams", C.c_int32),
        ("n_points", C.c_int32),
        ("n_obs", C.c_int32),
        ("cam_pose", _dp),
        ("cam_fixed", _u8p),
        ("points", _dp),
        ("point_fixed", _u8p),
        ("obs_uv", _dp),
        ("obs_cam", _i32p),
        ("obs_point", _i32p),
        ("camera_model", C.c_int32),
        ("reserved0", C.c_int32),
        ("intrinsics", C.c_double * 8),
    ]


class nav_ba_options(C.Structure):
    _fields_ = [
        ("iterations", C.c_int32),
        ("precision", C.c_int32),
        ("solver", C.c_int32),
        ("robust", C.c_int32),
        ("huber_delta", C.c_double),
        ("initial_lambda", C.c_double),
        ("tau", C.c_double),
        ("max_trials", C.c_int32),
        ("optimize_distortion", C.c_int32),
        ("pcg_tolerance", C.c_double),
        ("pcg_max_iterations", C.c_int32),
        ("deterministic", C.c_int32),
        ("reserved", C.c_int32 * 8),
    ]


class nav_ba_result(C.Structure):
    _fields_ = [
        ("cam_pose_out", _dp),
        ("points_out", _dp),
        ("intrinsics_out", _dp),
        ("cost_trace", _dp),
        ("initial_cost", C.c_double),
        ("final_cost", C.c_double),
        ("final_lambda", C.c_double),
        ("time_setup_ms", C.c_double),
        ("time_solve_ms", C.c_double),
        ("time_download_ms", C.c_double),
        ("iterations_done", C.c_int32),
        ("trials_accepted", C.c_int32),
        ("trials_rejected", C.c_int32),
        ("termination", C.c_int32),
        ("n_active_edges", C.c_int32),
        ("n_free_cams", C.c_int32),
        ("n_free_points", C.c_int32),
        ("n_schur_blocks", C.c_int32),
        ("pcg_iterations_total", C.c_int32),
        ("status", C.c_int32),
        ("edge_iterations", C.c_int64),
        ("h2d_bytes", C.c_int64),
        ("d2h_bytes", C.c_int64),
        ("n_depth_nonpositive", C.c_int32),
        ("reserved1", C.c_int32),
    ]


class nav_ba_pose_problem(C.Structure):
    _fields_ = [("n_obs", C.c_int32), ("camera_model", C.c_int32), ("pose", C.POINTER(C.c_double)),
                ("points", C.POINTER(C.c_double)), ("obs_uv", C.POINTER(C.c_double)), ("intrinsics", C.c_double * 8)]


class nav_ba_pose_result(C.Structure):
    _fields_ = [("pose_out", C.POINTER(C.c_double)), ("initial_cost", C.c_double), ("final_cost", C.c_double),
                ("final_lambda", C.c_double), ("iterations_done", C.c_int32), ("trials_accepted", C.c_int32),
                ("trials_rejected", C.c_int32), ("termination", C.c_int32), ("status", C.c_int32),
                ("n_depth_nonpositive", C.c_int32)]


@dataclass
class PoseProblem:
    """One motion-only problem: a pose against fixed world points (nav_ba_pose_problem)."""

    pose: np.ndarray          # (12,) row-major [R|t] of T_cw
    points: np.ndarray        # (n_obs, 3) world point of each observation
    obs_uv: np.ndarray        # (n_obs, 2)
    intrinsics: np.ndarray    # (8,)
    camera_model: int = CAM_PINHOLE

    def __post_init__(self):
        self.pose = np.ascontiguousarray(self.pose, np.float64).reshape(12)
        self.points = np.ascontiguousarray(self.points, np.float64).reshape(-1, 3)
        self.obs_uv = np.ascontiguousarray(self.obs_uv, np.float64).reshape(-1, 2)
        self.intrinsics = np.ascontiguousarray(self.intrinsics, np.float64).reshape(8)

    def as_c(self) -> nav_ba_pose_problem:
        p = nav_ba_pose_problem()
        p.n_obs = self.obs_uv.shape[0]
        p.camera_model = int(self.camera_model)
        p.pose = _ptr(self.pose, C.c_double)
        p.points = _ptr(self.points, C.c_double)
        p.obs_uv = _ptr(self.obs_uv, C.c_double)
        for i in range(8):
            p.intrinsics[i] = float(self.intrinsics[i])
        return p

    def as_problem(self) -> "Problem":
        """The same problem as a general one: one free camera, every point fixed."""
        n = self.obs_uv.shape[0]
        return Problem(cam_pose=self.pose.reshape(1, 12), points=self.points, obs_uv=self.obs_uv,
                       obs_cam=np.zeros(n, np.int32), obs_point=np.arange(n, dtype=np.int32),
                       intrinsics=self.intrinsics, cam_fixed=np.zeros(1, np.uint8),
                       point_fixed=np.ones(n, np.uint8), camera_model=self.camera_model)


class nav_ba_twoview(C.Structure):
    _fields_ = [("n_matches", C.c_int32), ("n_hyp", C.c_int32), ("K", C.c_double * 4),
                ("kp1", C.POINTER(C.c_double)), ("kp2", C.POINTER(C.c_double)), ("inlier", C.POINTER(C.c_uint8)),
                ("R", C.POINTER(C.c_double)), ("t", C.POINTER(C.c_double)), ("th2", C.c_double),
                ("min_parallax_cos", C.c_double), ("min_triangulated", C.c_int32), ("reserved", C.c_int32)]


class nav_ba_twoview_result(C.Structure):
    _fields_ = [("points", C.POINTER(C.c_double)), ("triangulated", C.POINTER(C.c_uint8)),
                ("good", C.POINTER(C.c_uint8)), ("n_good", C.POINTER(C.c_int32)),
                ("parallax_deg", C.POINTER(C.c_double))]


VJP_MAX_STEPS = 64


class nav_ba_schedule(C.Structure):
    _fields_ = [("replay", C.c_int32), ("n_steps", C.c_int32), ("lam", C.c_double * VJP_MAX_STEPS)]

    @property
    def lambdas(self) -> list[float]:
        return [self.lam[i] for i in range(self.n_steps)]

    @staticmethod
    def of(lambdas, replay: bool = True) -> "nav_ba_schedule":
        s = nav_ba_schedule()
        s.replay = 1 if replay else 0
        s.n_steps = len(lambdas)
        for i, v in enumerate(lambdas):
            s.lam[i] = float(v)
        return s


class nav_ba_cotangent(C.Structure):
    _fields_ = [("cost", C.c_double), ("cam_pose", C.POINTER(C.c_double)), ("points", C.POINTER(C.c_double))]


class nav_ba_grads(C.Structure):
    _fields_ = [("obs_uv", C.POINTER(C.c_double)), ("intrinsics", C.c_double * 8),
                ("cam_tangent", C.POINTER(C.c_double)), ("points", C.POINTER(C.c_double))]


class nav_synth_params(C.Structure):
    _fields_ = [
        ("family", C.c_int32),
        ("n_cams", C.c_int32),
        ("n_points", C.c_int32),
        ("n_windows", C.c_int32),
        ("seed", C.c_uint64),
        ("pixel_noise", C.c_double),
        ("outlier_frac", C.c_double),
        ("rot_perturb", C.c_double),
        ("trans_perturb", C.c_double),
        ("point_perturb", C.c_double),
        ("min_cams", C.c_int32),
        ("min_points", C.c_int32),
    ]


HUBER_DELTA_NAV24 = float(np.float32(np.sqrt(5.99)))  # BE_GraphOptim.cpp:125 (float threshold)


def default_options(**kw) -> nav_ba_options:
    """Defaults of nav24's PR_VBA call (Problem.hpp:84, :112; BE_GraphOptim.cpp:125)."""
    o = nav_ba_options()
    o.iterations = 5
    o.precision = FP64
    o.solver = SOLVER_CHOLESKY
    o.robust = 0
    o.huber_delta = HUBER_DELTA_NAV24
    o.initial_lambda = 0.0
    o.tau = 1e-5
    o.max_trials = 10
    o.optimize_distortion = 0
    o.pcg_tolerance = 1e-6
    o.pcg_max_iterations = 100
    o.deterministic = 1
    for k, v in kw.items():
        if not hasattr(o, k):
            raise AttributeError(k)
        setattr(o, k, v)
    return o


def _ptr(a: np.ndarray | None, ctype):
    if a is None:
        return C.cast(None, C.POINTER(ctype))
    return a.ctypes.data_as(C.POINTER(ctype))


@dataclass
class Problem:
    """A BA problem as numpy arrays (the flattened PR_VBA of include/nav_ba.h)."""

    cam_pose: np.ndarray                 # (n_cams, 12) float64, row-major [R|t] of T_cw
    points: np.ndarray                   # (n_points, 3) float64
    obs_uv: np.ndarray                   # (n_obs, 2) float64
    obs_cam: np.ndarray                  # (n_obs,) int32
    obs_point: np.ndarray                # (n_obs,) int32
    intrinsics: np.ndarray               # (8,) float64
    cam_fixed: np.ndarray | None = None  # (n_cams,) uint8
    point_fixed: np.ndarray | None = None
    camera_model: int = CAM_PINHOLE
    _keep: list = field(default_factory=list, repr=False)

    def __post_init__(self):
        self.cam_pose = np.ascontiguousarray(self.cam_pose, dtype=np.float64).reshape(-1, 12)
        self.points = np.ascontiguousarray(self.points, dtype=np.float64).reshape(-1, 3)
        self.obs_uv = np.ascontiguousarray(self.obs_uv, dtype=np.float64).reshape(-1, 2)
        self.obs_cam = np.ascontiguousarray(self.obs_cam, dtype=np.int32).reshape(-1)
        self.obs_point = np.ascontiguousarray(self.obs_point, dtype=np.int32).reshape(-1)
        self.intrinsics = np.ascontiguousarray(self.intrinsics, dtype=np.float64).reshape(8)
        if self.cam_fixed is not None:
            self.cam_fixed = np.ascontiguousarray(self.cam_fixed, dtype=np.uint8).reshape(-1)
        if self.point_fixed is not None:
            self.point_fixed = np.ascontiguousarray(self.point_fixed, dtype=np.uint8).reshape(-1)

    @property
    def n_cams(self):
        return self.cam_pose.shape[0]

    @property
    def n_points(self):
        return self.points.shape[0]

    @property
    def n_obs(self):
        return self.obs_uv.shape[0]

    def as_c(self) -> nav_ba_problem:
        p = nav_ba_problem()
        p.n_cams = self.n_cams
        p.n_points = self.n_points
        p.n_obs = self.n_obs
        p.cam_pose = _ptr(self.cam_pose, C.c_double)
        p.cam_fixed = _ptr(self.cam_fixed, C.c_uint8)
        p.points = _ptr(self.points, C.c_double)
        p.point_fixed = _ptr(self.point_fixed, C.c_uint8)
        p.obs_uv = _ptr(self.obs_uv, C.c_double)
        p.obs_cam = _ptr(self.obs_cam, C.c_int32)
        p.obs_point = _ptr(self.obs_point, C.c_int32)
        p.camera_model = int(self.camera_model)
        for i in range(8):
            p.intrinsics[i] = float(self.intrinsics[i])
        return p

    def copy(self) -> "Problem":
        return Problem(
            self.cam_pose.copy(), self.points.copy(), self.obs_uv.copy(), self.obs_cam.copy(),
            self.obs_point.copy(), self.intrinsics.copy(),
            None if self.cam_fixed is None else self.cam_fixed.copy(),
            None if self.point_fixed is None else self.point_fixed.copy(), self.camera_model)


@dataclass
class Result:
    status: int
    cam_pose: np.ndarray
    points: np.ndarray
    intrinsics: np.ndarray
    cost_trace: np.ndarray
    stats: dict


class ResultBuffers:
    """Host output buffers for one nav_ba_result."""

    def __init__(self, prob: Problem, iterations: int):
        self.cam_pose = np.zeros((prob.n_cams, 12), np.float64)
        self.points = np.zeros((prob.n_points, 3), np.float64)
        self.intrinsics = np.zeros(8, np.float64)
        self.cost_trace = np.full(iterations + 1, np.nan, np.float64)
        self.c = nav_ba_result()
        self.c.cam_pose_out = _ptr(self.cam_pose, C.c_double)
        self.c.points_out = _ptr(self.points, C.c_double)
        self.c.intrinsics_out = _ptr(self.intrinsics, C.c_double)
        self.c.cost_trace = _ptr(self.cost_trace, C.c_double)

    def result(self, status: int) -> Result:
        r = self.c
        stats = {name: getattr(r, name) for name, _ in nav_ba_result._fields_
                 if name not in ("cam_pose_out", "points_out", "intrinsics_out", "cost_trace")}
        n = max(0, r.iterations_done) + 1
        return Result(status, self.cam_pose, self.points, self.intrinsics, self.cost_trace[:n].copy(), stats)
