"""ctypes bindings of the CPU oracle (test infrastructure only; see ba_oracle.cpp's header)."""
from __future__ import annotations

import ctypes as C

import numpy as np

from nav24_gb300 import abi

from .build import build

_LIB = None


def lib():
    global _LIB
    if _LIB is None:
        L = C.CDLL(str(build()))
        P, O, R = C.POINTER(abi.nav_ba_problem), C.POINTER(abi.nav_ba_options), C.POINTER(abi.nav_ba_result)
        dp = C.POINTER(C.c_double)
        L.oracle_solve.argtypes = [P, O, R, C.c_int32]
        L.oracle_solve.restype = C.c_int32
        L.oracle_solve_schedule.argtypes = [P, O, R, C.c_int32, C.POINTER(abi.nav_ba_schedule)]
        L.oracle_solve_schedule.restype = C.c_int32
        L.oracle_linearize.argtypes = [P, O, dp, dp, dp, dp]
        L.oracle_linearize.restype = C.c_int32
        L.oracle_linearize_mode.argtypes = [P, O, C.c_int32, dp, dp, dp, dp]
        L.oracle_linearize_mode.restype = C.c_int32
        L.oracle_distortion_jacobian.argtypes = [P, dp]
        L.oracle_distortion_jacobian.restype = C.c_int32
        L.oracle_reduced_system.argtypes = [P, O, C.c_double, C.c_int32, C.POINTER(C.c_int32), dp, dp,
                                            C.POINTER(C.c_int32)]
        L.oracle_reduced_system.restype = C.c_int32
        L.oracle_cost.argtypes = [P, O, dp]
        L.oracle_cost.restype = C.c_int32
        L.oracle_se3_update.argtypes = [dp, dp, dp]
        L.oracle_pose_roundtrip.argtypes = [dp, dp]
        _LIB = L
    return _LIB


def _d(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def solve(prob: abi.Problem, opt: abi.nav_ba_options, n_threads: int = 1) -> abi.Result:
    buf = abi.ResultBuffers(prob, opt.iterations)
    p = prob.as_c()
    st = lib().oracle_solve(C.byref(p), C.byref(opt), C.byref(buf.c), n_threads)
    return buf.result(st)


def solve_schedule(prob: abi.Problem, opt: abi.nav_ba_options, lambdas=None, n_threads: int = 1):
    """Record (lambdas None) or replay the damping schedule; returns (Result, lambdas)."""
    replay = lambdas is not None
    sched = abi.nav_ba_schedule.of(lambdas if replay else [], replay)
    buf = abi.ResultBuffers(prob, max(opt.iterations, len(lambdas) if replay else 0))
    p = prob.as_c()
    st = lib().oracle_solve_schedule(C.byref(p), C.byref(opt), C.byref(buf.c), n_threads, C.byref(sched))
    return buf.result(st), sched.lambdas


def linearize(prob: abi.Problem, opt: abi.nav_ba_options, reference_rounding: bool = False):
    """Residuals, Jacobians and robust weights of every observation.  reference_rounding: the
    Kannala-Brandt 8 model with the reference's own float roundings (oracle_linearize_mode 1)."""
    n = prob.n_obs
    e, jc, jp, w = (np.zeros((n, 2)), np.zeros((n, 2, 6)), np.zeros((n, 2, 3)), np.zeros(n))
    p = prob.as_c()
    st = lib().oracle_linearize_mode(C.byref(p), C.byref(opt), 1 if reference_rounding else 0, _d(e), _d(jc),
                                     _d(jp), _d(w))
    if st != abi.OK:
        raise RuntimeError(f"oracle_linearize status {st}")
    return e, jc, jp, w


def distortion_jacobian(prob: abi.Problem):
    jk = np.zeros((prob.n_obs, 2, 2))
    p = prob.as_c()
    st = lib().oracle_distortion_jacobian(C.byref(p), _d(jk))
    if st != abi.OK:
        raise RuntimeError(f"oracle_distortion_jacobian status {st}")
    return jk


def reduced_system(prob: abi.Problem, opt: abi.nav_ba_options, lam: float):
    p = prob.as_c()
    nf = C.c_int32()
    idx = np.zeros(prob.n_cams, np.int32)
    L = lib()
    L.oracle_reduced_system(C.byref(p), C.byref(opt), lam, 0, C.byref(nf), None, None,
                            idx.ctypes.data_as(C.POINTER(C.c_int32)))
    n = 6 * nf.value
    S, b = np.zeros((n, n)), np.zeros(n)
    st = L.oracle_reduced_system(C.byref(p), C.byref(opt), lam, nf.value, C.byref(nf), _d(S), _d(b),
                                 idx.ctypes.data_as(C.POINTER(C.c_int32)))
    if st != abi.OK:
        raise RuntimeError(f"oracle_reduced_system status {st}")
    return S, b, idx


def cost(prob: abi.Problem, opt: abi.nav_ba_options) -> float:
    p = prob.as_c()
    c = C.c_double()
    st = lib().oracle_cost(C.byref(p), C.byref(opt), C.byref(c))
    if st != abi.OK:
        raise RuntimeError(f"oracle_cost status {st}")
    return c.value


def se3_update(pose12, delta6):
    pose12 = np.ascontiguousarray(pose12, np.float64)
    delta6 = np.ascontiguousarray(delta6, np.float64)
    out = np.zeros(12)
    lib().oracle_se3_update(_d(pose12), _d(delta6), _d(out))
    return out


def pose_roundtrip(pose12):
    pose12 = np.ascontiguousarray(pose12, np.float64)
    out = np.zeros(12)
    lib().oracle_pose_roundtrip(_d(pose12), _d(out))
    return out
