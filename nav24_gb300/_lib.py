"""ctypes binding of libnavba.so (the product C ABI, include/nav_ba.h).

The library is built in-tree (nav24_gb300/_build).  Loading fails loudly when it is missing:
there is no CPU fallback for any entry point.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

from . import abi

LIB_PATH = Path(__file__).resolve().parent / "_build" / "libnavba.so"

# Every entry point declared in include/nav_ba.h.
EXPORTS = [
    "nav_ba_options_default", "nav_ba_create", "nav_ba_destroy", "nav_ba_solve",
    "nav_ba_solve_batched", "nav_ba_prepare", "nav_ba_run", "nav_ba_fetch", "nav_ba_prepare_batched",
    "nav_ba_fetch_batched", "nav_ba_linearize",
    "nav_ba_reduced_system", "nav_ba_cost", "nav_ba_last_error", "nav_ba_status_string",
    "nav_ba_abi_version", "nav_ba_solve_noalloc", "nav_ba_vjp", "nav_ba_solve_pose_batched",
    "nav_ba_twoview_check", "nav_ba_undistort_points",
]

_LIB = None


class NativeLibraryMissing(RuntimeError):
    pass


def load(path: os.PathLike | None = None) -> C.CDLL:
    """Load libnavba.so and declare its signatures (raises if the library is absent)."""
    global _LIB
    if _LIB is not None and path is None:
        return _LIB
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise NativeLibraryMissing(f"{p} is missing: build it with nav24_gb300.build.build_product()")
    L = C.CDLL(str(p))
    P, O, R = C.POINTER(abi.nav_ba_problem), C.POINTER(abi.nav_ba_options), C.POINTER(abi.nav_ba_result)
    dp, ip = C.POINTER(C.c_double), C.POINTER(C.c_int32)
    ctxp = C.c_void_p
    L.nav_ba_options_default.argtypes = [O]
    L.nav_ba_options_default.restype = None
    L.nav_ba_create.argtypes = [C.POINTER(ctxp), C.c_int32]
    L.nav_ba_create.restype = C.c_int
    L.nav_ba_destroy.argtypes = [ctxp]
    L.nav_ba_destroy.restype = None
    L.nav_ba_solve.argtypes = [ctxp, P, O, R]
    L.nav_ba_solve.restype = C.c_int
    L.nav_ba_solve_batched.argtypes = [ctxp, P, C.c_int32, O, R]
    L.nav_ba_solve_batched.restype = C.c_int
    L.nav_ba_prepare.argtypes = [ctxp, P, O]
    L.nav_ba_prepare.restype = C.c_int
    L.nav_ba_run.argtypes = [ctxp, O, R]
    L.nav_ba_run.restype = C.c_int
    L.nav_ba_fetch.argtypes = [ctxp, R]
    L.nav_ba_fetch.restype = C.c_int
    L.nav_ba_prepare_batched.argtypes = [ctxp, P, C.c_int32, O]
    L.nav_ba_prepare_batched.restype = C.c_int
    L.nav_ba_fetch_batched.argtypes = [ctxp, R]
    L.nav_ba_fetch_batched.restype = C.c_int
    L.nav_ba_linearize.argtypes = [ctxp, P, O, dp, dp, dp, dp]
    L.nav_ba_linearize.restype = C.c_int
    L.nav_ba_reduced_system.argtypes = [ctxp, P, O, C.c_double, C.c_int32, ip, dp, dp, ip]
    L.nav_ba_reduced_system.restype = C.c_int
    L.nav_ba_cost.argtypes = [ctxp, P, O, dp]
    L.nav_ba_cost.restype = C.c_int
    L.nav_ba_last_error.argtypes = [ctxp]
    L.nav_ba_last_error.restype = C.c_char_p
    L.nav_ba_status_string.argtypes = [C.c_int]
    L.nav_ba_status_string.restype = C.c_char_p
    L.nav_ba_solve_noalloc.argtypes = [ctxp, P, O, R]
    L.nav_ba_solve_noalloc.restype = C.c_int
    L.nav_ba_vjp.argtypes = [ctxp, P, O, C.POINTER(abi.nav_ba_schedule), C.POINTER(abi.nav_ba_cotangent), R,
                             C.POINTER(abi.nav_ba_grads)]
    L.nav_ba_vjp.restype = C.c_int
    L.nav_ba_solve_pose_batched.argtypes = [ctxp, C.POINTER(abi.nav_ba_pose_problem), C.c_int32, O,
                                            C.POINTER(abi.nav_ba_pose_result)]
    L.nav_ba_solve_pose_batched.restype = C.c_int
    L.nav_ba_twoview_check.argtypes = [ctxp, C.POINTER(abi.nav_ba_twoview), C.POINTER(abi.nav_ba_twoview_result)]
    L.nav_ba_twoview_check.restype = C.c_int
    L.nav_ba_undistort_points.argtypes = [ctxp, dp, dp, C.c_int32, C.c_int32, dp, dp]
    L.nav_ba_undistort_points.restype = C.c_int
    L.nav_ba_abi_version.argtypes = []
    L.nav_ba_abi_version.restype = C.c_int32
    if path is None:
        _LIB = L
    return L


def _d(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class BAError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"status {status}: {msg}")
        self.status = status


class Context:
    """One nav_ba_ctx (one CUDA stream on one device)."""

    def __init__(self, device: int = 0):
        self.L = load()
        h = C.c_void_p()
        st = self.L.nav_ba_create(C.byref(h), device)
        if st != abi.OK:
            raise BAError(st, self.L.nav_ba_status_string(st).decode())
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.L.nav_ba_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def last_error(self) -> str:
        return self.L.nav_ba_last_error(self.h).decode()

    def _check(self, st: int, ok=(abi.OK,)):
        if st not in ok:
            raise BAError(st, self.last_error() or self.L.nav_ba_status_string(st).decode())
        return st

    def solve(self, prob: abi.Problem, opt: abi.nav_ba_options, raise_on_error=True) -> abi.Result:
        buf = abi.ResultBuffers(prob, opt.iterations)
        p = prob.as_c()
        st = self.L.nav_ba_solve(self.h, C.byref(p), C.byref(opt), C.byref(buf.c))
        if raise_on_error:
            self._check(st, (abi.OK, abi.EMPTY))
        return buf.result(st)

    def solve_noalloc(self, prob: abi.Problem, opt: abi.nav_ba_options, raise_on_error=True) -> abi.Result:
        """nav_ba_solve_noalloc: one window solved in the library's static device array."""
        buf = abi.ResultBuffers(prob, opt.iterations)
        p = prob.as_c()
        st = self.L.nav_ba_solve_noalloc(self.h, C.byref(p), C.byref(opt), C.byref(buf.c))
        if raise_on_error:
            self._check(st, (abi.OK, abi.EMPTY))
        return buf.result(st)

    def vjp(self, prob: abi.Problem, opt: abi.nav_ba_options, lambdas=None, cost_bar: float | None = None,
            pose_bar: np.ndarray | None = None, point_bar: np.ndarray | None = None):
        """nav_ba_vjp.  lambdas None: run LM and record the accepted steps' damping; else replay
        those steps.  With any cotangent given (cost_bar, pose_bar [n_cams, 12], point_bar
        [n_points, 3]) the backward runs too.  Returns (Result, lambdas, grads or None), grads a
        dict of obs_uv [n_obs, 2], intrinsics [4] (fx, fy, cx, cy), cam_tangent [n_cams, 6] and
        points [n_points, 3]."""
        replay = lambdas is not None
        sched = abi.nav_ba_schedule.of(lambdas if replay else [], replay)
        buf = abi.ResultBuffers(prob, max(opt.iterations, len(lambdas) if replay else 0))
        p = prob.as_c()
        bwd = cost_bar is not None or pose_bar is not None or point_bar is not None
        cot = grads = None
        keep = []
        if bwd:
            cot = abi.nav_ba_cotangent()
            cot.cost = 0.0 if cost_bar is None else float(cost_bar)
            if pose_bar is not None:
                pb = np.ascontiguousarray(pose_bar, np.float64).reshape(prob.n_cams, 12)
                keep.append(pb)
                cot.cam_pose = _d(pb)
            if point_bar is not None:
                qb = np.ascontiguousarray(point_bar, np.float64).reshape(prob.n_points, 3)
                keep.append(qb)
                cot.points = _d(qb)
            g = {"obs_uv": np.zeros((prob.n_obs, 2)), "cam_tangent": np.zeros((prob.n_cams, 6)),
                 "points": np.zeros((prob.n_points, 3))}
            grads = abi.nav_ba_grads()
            grads.obs_uv = _d(g["obs_uv"])
            grads.cam_tangent = _d(g["cam_tangent"])
            grads.points = _d(g["points"])
        st = self.L.nav_ba_vjp(self.h, C.byref(p), C.byref(opt), C.byref(sched),
                               C.byref(cot) if bwd else None, C.byref(buf.c), C.byref(grads) if bwd else None)
        self._check(st, (abi.OK, abi.EMPTY))
        out = None
        if bwd:
            g["intrinsics"] = np.array([grads.intrinsics[i] for i in range(4)])
            out = g
        return buf.result(st), sched.lambdas, out

    def solve_pose_batched(self, probs: list[abi.PoseProblem], opt: abi.nav_ba_options):
        """nav_ba_solve_pose_batched: motion-only BA of every problem in one launch.  Returns
        [(pose [12], stats dict)]."""
        n = len(probs)
        cp = (abi.nav_ba_pose_problem * max(n, 1))(*[p.as_c() for p in probs])
        outs = [np.zeros(12) for _ in probs]
        cr = (abi.nav_ba_pose_result * max(n, 1))()
        for i in range(n):
            cr[i].pose_out = _d(outs[i])
        st = self.L.nav_ba_solve_pose_batched(self.h, cp, n, C.byref(opt), cr)
        self._check(st)
        return [(outs[i], {f: getattr(cr[i], f) for f, _ in abi.nav_ba_pose_result._fields_ if f != "pose_out"})
                for i in range(n)]

    def twoview_check(self, K, kp1, kp2, R, t, th2: float, min_parallax_cos: float, min_triangulated: int = 50,
                      inlier=None):
        """nav_ba_twoview_check for hypotheses R [n_hyp, 3, 3], t [n_hyp, 3].  Returns a dict of points
        [n_hyp, n, 3], triangulated / good [n_hyp, n] (bool), n_good [n_hyp], parallax_deg [n_hyp]."""
        kp1 = np.ascontiguousarray(kp1, np.float64).reshape(-1, 2)
        kp2 = np.ascontiguousarray(kp2, np.float64).reshape(-1, 2)
        R = np.ascontiguousarray(R, np.float64).reshape(-1, 9)
        t = np.ascontiguousarray(t, np.float64).reshape(-1, 3)
        n, nh = kp1.shape[0], R.shape[0]
        tv = abi.nav_ba_twoview()
        tv.n_matches, tv.n_hyp = n, nh
        for i in range(4):
            tv.K[i] = float(K[i])
        tv.kp1, tv.kp2, tv.R, tv.t = _d(kp1), _d(kp2), _d(R), _d(t)
        inl = None
        if inlier is not None:
            inl = np.ascontiguousarray(inlier, np.uint8)
            tv.inlier = inl.ctypes.data_as(C.POINTER(C.c_uint8))
        tv.th2, tv.min_parallax_cos, tv.min_triangulated = th2, min_parallax_cos, min_triangulated
        out = {"points": np.zeros((nh, n, 3)), "triangulated": np.zeros((nh, n), np.uint8),
               "good": np.zeros((nh, n), np.uint8), "n_good": np.zeros(nh, np.int32), "parallax_deg": np.zeros(nh)}
        r = abi.nav_ba_twoview_result()
        r.points = _d(out["points"])
        r.triangulated = out["triangulated"].ctypes.data_as(C.POINTER(C.c_uint8))
        r.good = out["good"].ctypes.data_as(C.POINTER(C.c_uint8))
        r.n_good = out["n_good"].ctypes.data_as(C.POINTER(C.c_int32))
        r.parallax_deg = _d(out["parallax_deg"])
        self._check(self.L.nav_ba_twoview_check(self.h, C.byref(tv), C.byref(r)))
        out["triangulated"] = out["triangulated"].astype(bool)
        out["good"] = out["good"].astype(bool)
        return out

    def undistort_points(self, K, dist, uv, iterations: int = 5) -> np.ndarray:
        """nav_ba_undistort_points: radial-tangential keypoint undistortion (returns [n, 2])."""
        Kd = np.ascontiguousarray(K, np.float64).reshape(4)
        dd = np.ascontiguousarray(dist, np.float64).reshape(4)
        uv = np.ascontiguousarray(uv, np.float64).reshape(-1, 2)
        out = np.empty_like(uv)
        self._check(self.L.nav_ba_undistort_points(self.h, _d(Kd), _d(dd), iterations, uv.shape[0], _d(uv), _d(out)))
        return out

    def solve_batched(self, probs: list[abi.Problem], opt: abi.nav_ba_options) -> list[abi.Result]:
        n = len(probs)
        cp = (abi.nav_ba_problem * n)(*[p.as_c() for p in probs])
        bufs = [abi.ResultBuffers(p, opt.iterations) for p in probs]
        cr = (abi.nav_ba_result * n)(*[b.c for b in bufs])
        st = self.L.nav_ba_solve_batched(self.h, cp, n, C.byref(opt), cr)
        self._check(st)
        out = []
        for b, r in zip(bufs, cr):
            b.c = r
            out.append(b.result(r.status))
        return out

    def batched_call(self, probs: list[abi.Problem], opt: abi.nav_ba_options) -> "BatchedCall":
        """A nav_ba_solve_batched call with its C structs and host output buffers built once, so
        that repeated calls time the C ABI alone."""
        return BatchedCall(self, probs, opt)

    def pose_call(self, probs: list[abi.PoseProblem], opt: abi.nav_ba_options) -> "PoseCall":
        """A nav_ba_solve_pose_batched call with its C structs and host output buffers built once,
        so that repeated calls time the C ABI alone."""
        return PoseCall(self, probs, opt)

    def prepare(self, prob: abi.Problem, opt: abi.nav_ba_options):
        self._prepared = prob  # keep the arrays alive
        p = prob.as_c()
        self._check(self.L.nav_ba_prepare(self.h, C.byref(p), C.byref(opt)))

    def prepare_batched(self, probs: list[abi.Problem], opt: abi.nav_ba_options):
        self._prepared_batch = probs
        n = len(probs)
        self._cp = (abi.nav_ba_problem * n)(*[p.as_c() for p in probs])
        self._check(self.L.nav_ba_prepare_batched(self.h, self._cp, n, C.byref(opt)))

    def fetch_batched(self, opt: abi.nav_ba_options) -> list[abi.Result]:
        probs = self._prepared_batch
        n = len(probs)
        bufs = [abi.ResultBuffers(p, opt.iterations) for p in probs]
        cr = (abi.nav_ba_result * n)(*[b.c for b in bufs])
        self._check(self.L.nav_ba_fetch_batched(self.h, cr))
        out = []
        for b, r in zip(bufs, cr):
            b.c = r
            out.append(b.result(r.status))
        return out

    def run(self, opt: abi.nav_ba_options) -> dict:
        r = abi.nav_ba_result()
        self._check(self.L.nav_ba_run(self.h, C.byref(opt), C.byref(r)))
        return {name: getattr(r, name) for name, _ in abi.nav_ba_result._fields_
                if name not in ("cam_pose_out", "points_out", "intrinsics_out", "cost_trace")}

    def fetch(self, opt: abi.nav_ba_options) -> abi.Result:
        buf = abi.ResultBuffers(self._prepared, opt.iterations)
        st = self.L.nav_ba_fetch(self.h, C.byref(buf.c))
        self._check(st)
        return buf.result(st)

    def linearize(self, prob: abi.Problem, opt: abi.nav_ba_options):
        n = prob.n_obs
        e, jc, jp, w = (np.zeros((n, 2)), np.zeros((n, 2, 6)), np.zeros((n, 2, 3)), np.zeros(n))
        p = prob.as_c()
        self._check(self.L.nav_ba_linearize(self.h, C.byref(p), C.byref(opt), _d(e), _d(jc), _d(jp), _d(w)))
        return e, jc, jp, w

    def reduced_system(self, prob: abi.Problem, opt: abi.nav_ba_options, lam: float):
        p = prob.as_c()
        nf = C.c_int32()
        idx = np.zeros(max(1, prob.n_cams), np.int32)
        ip = idx.ctypes.data_as(C.POINTER(C.c_int32))
        self._check(self.L.nav_ba_reduced_system(self.h, C.byref(p), C.byref(opt), lam, 0, C.byref(nf), None, None, ip))
        n = 6 * nf.value
        S, b = np.zeros((n, n)), np.zeros(n)
        self._check(self.L.nav_ba_reduced_system(self.h, C.byref(p), C.byref(opt), lam, nf.value, C.byref(nf),
                                                 _d(S), _d(b), ip))
        return S, b, idx[: prob.n_cams]

    def cost(self, prob: abi.Problem, opt: abi.nav_ba_options) -> float:
        p = prob.as_c()
        c = C.c_double()
        self._check(self.L.nav_ba_cost(self.h, C.byref(p), C.byref(opt), C.byref(c)))
        return c.value


class BatchedCall:
    def __init__(self, ctx: Context, probs: list[abi.Problem], opt: abi.nav_ba_options):
        self.ctx, self.probs, self.opt = ctx, probs, opt
        n = len(probs)
        self.n = n
        self.cp = (abi.nav_ba_problem * n)(*[p.as_c() for p in probs])
        self.bufs = [abi.ResultBuffers(p, opt.iterations) for p in probs]
        self.cr = (abi.nav_ba_result * n)(*[b.c for b in self.bufs])

    def __call__(self) -> int:
        return self.ctx._check(self.ctx.L.nav_ba_solve_batched(self.ctx.h, self.cp, self.n, C.byref(self.opt), self.cr))

    def results(self) -> list[abi.Result]:
        out = []
        for b, r in zip(self.bufs, self.cr):
            b.c = r
            out.append(b.result(r.status))
        return out


class PoseCall:
    def __init__(self, ctx: Context, probs: list[abi.PoseProblem], opt: abi.nav_ba_options):
        self.ctx, self.probs, self.opt = ctx, probs, opt
        n = len(probs)
        self.n = n
        self.cp = (abi.nav_ba_pose_problem * max(n, 1))(*[p.as_c() for p in probs])
        self.outs = [np.zeros(12) for _ in probs]
        self.cr = (abi.nav_ba_pose_result * max(n, 1))()
        for i in range(n):
            self.cr[i].pose_out = _d(self.outs[i])

    def __call__(self) -> int:
        return self.ctx._check(self.ctx.L.nav_ba_solve_pose_batched(self.ctx.h, self.cp, self.n, C.byref(self.opt),
                                                                    self.cr))

    def results(self):
        return [(self.outs[i], {f: getattr(self.cr[i], f) for f, _ in abi.nav_ba_pose_result._fields_
                                if f != "pose_out"}) for i in range(self.n)]
