"""ctypes bindings of oracle/_ref/libnav24ref.so: nav24's own edge and camera-model code compiled
from the reference tree (TEST INFRASTRUCTURE; built by oracle/ref_build.py).  Only the tests and
the fixture generator tests/golden/make_ref_vectors.py load it, and only where the reference tree
exists; elsewhere the committed vectors stand in for it."""
from __future__ import annotations

import ctypes as C

import numpy as np

from nav24_gb300 import abi

from .ref_build import build

_LIB = None


def lib():
    """The reference library, or None when the reference tree is absent."""
    global _LIB
    if _LIB is None:
        path = build()
        if path is None:
            return None
        L = C.CDLL(str(path))
        P, dp = C.POINTER(abi.nav_ba_problem), C.POINTER(C.c_double)
        L.ref_edges.argtypes = [P, dp, dp, dp, C.POINTER(C.c_uint8)]
        L.ref_edges.restype = C.c_int32
        L.ref_project.argtypes = [P, C.c_int32, dp, dp, dp]
        L.ref_project.restype = C.c_int32
        _LIB = L
    return _LIB


def _d(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def edges(prob: abi.Problem):
    """(e [n, 2], jc [n, 2, 6], jp [n, 2, 3], depth_positive [n]) from nav24's EdgeSE3ProjectXYZ."""
    n = prob.n_obs
    e, jc, jp = np.zeros((n, 2)), np.zeros((n, 2, 6)), np.zeros((n, 2, 3))
    dpos = np.zeros(n, np.uint8)
    p = prob.as_c()
    st = lib().ref_edges(C.byref(p), _d(e), _d(jc), _d(jp), dpos.ctypes.data_as(C.POINTER(C.c_uint8)))
    if st != abi.OK:
        raise RuntimeError(f"ref_edges status {st}")
    return e, jc, jp, dpos


def project(prob: abi.Problem, xc: np.ndarray):
    """(uv [n, 2], jac [n, 2, 3]) of camera-frame points through nav24's Calibration."""
    xc = np.ascontiguousarray(xc, np.float64).reshape(-1, 3)
    n = xc.shape[0]
    uv, jac = np.zeros((n, 2)), np.zeros((n, 2, 3))
    p = prob.as_c()
    st = lib().ref_project(C.byref(p), n, _d(xc), _d(uv), _d(jac))
    if st != abi.OK:
        raise RuntimeError(f"ref_project status {st}")
    return uv, jac
