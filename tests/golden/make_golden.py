"""Generate the golden vectors under tests/golden/.

    python tests/golden/make_golden.py

known_answer.json
    Residuals and Jacobians of single edges derived symbolically with sympy, independently of
    the oracle's closed forms: e(d_pose, d_point) = z - pi(exp(d_pose) (R (X + d_point) + t)) is
    built from the SE(3) exponential (series of the Rodrigues coefficients, exact for first
    derivatives at 0) and differentiated exactly in rational arithmetic.  pi is nav24's pinhole
    projection (core/sensor/camera/models/Pinhole.cpp:30-36) or the pinhole with the radial factor
    1 + k1 r^2 + k2 r^4.  The pose twist is ordered [omega; upsilon] (rotation first), the order
    of the reference's SE3deriv (core/dataTypes/optimization/OptimizableTypes.cpp:155-158).

ring_fixture.npz
    The ring workload (family 0, seed 1000: 10 cameras, 500 points, camera 0 fixed) as input
    arrays, with the oracle's 10-iteration solve (lambda0 = 1e-3) as a regression pin.

synth_digests.json
    SHA-256 digests of small instances of every workload family (SYNTH_CASES): the generator is
    host-independent, so the same digests must come out on x86-64 and aarch64.
"""
from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np
import sympy as sp

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))


def rot_from_int_quat(w, x, y, z):
    n = w * w + x * x + y * y + z * z
    M = sp.Matrix([
        [w * w + x * x - y * y - z * z, 2 * (x * y - w * z), 2 * (x * z + w * y)],
        [2 * (x * y + w * z), w * w - x * x + y * y - z * z, 2 * (y * z - w * x)],
        [2 * (x * z - w * y), 2 * (y * z + w * x), w * w - x * x - y * y + z * z],
    ])
    return M / n


def edge_known_answer(case):
    w = sp.symbols("w0:3")
    u = sp.symbols("u0:3")
    d = sp.symbols("d0:3")
    R = rot_from_int_quat(*case["quat_wxyz"])
    t = sp.Matrix([sp.Rational(v) for v in case["t"]])
    X = sp.Matrix([sp.Rational(v) for v in case["X"]])
    z = [sp.Rational(v) for v in case["z"]]
    fx, fy, cx, cy = (sp.Rational(v) for v in case["fx_fy_cx_cy"])
    k1, k2 = (sp.Rational(v) for v in case.get("k1_k2", ["0", "0"]))
    W = sp.Matrix([[0, -w[2], w[1]], [w[2], 0, -w[0]], [-w[1], w[0], 0]])
    th2 = w[0] ** 2 + w[1] ** 2 + w[2] ** 2
    a = 1 - th2 / 6 + th2 ** 2 / 120
    b = sp.Rational(1, 2) - th2 / 24 + th2 ** 2 / 720
    c = sp.Rational(1, 6) - th2 / 120 + th2 ** 2 / 5040
    I3 = sp.eye(3)
    Rw = I3 + a * W + b * W * W
    Vw = I3 + b * W + c * W * W
    Y = R * (X + sp.Matrix(d)) + t
    Yc = Rw * Y + Vw * sp.Matrix(u)
    xn, yn = Yc[0] / Yc[2], Yc[1] / Yc[2]
    r2 = xn ** 2 + yn ** 2
    dist = 1 + k1 * r2 + k2 * r2 ** 2
    e = sp.Matrix([z[0] - (fx * dist * xn + cx), z[1] - (fy * dist * yn + cy)])
    zero = {s: 0 for s in (*w, *u, *d)}
    e0 = [e[i].subs(zero) for i in range(2)]
    jc = [[sp.diff(e[i], v).subs(zero) for v in (*w, *u)] for i in range(2)]
    jp = [[sp.diff(e[i], v).subs(zero) for v in d] for i in range(2)]
    Rn = [[float(R[i, j]) for j in range(3)] for i in range(3)]
    pose12 = [Rn[0][0], Rn[0][1], Rn[0][2], float(t[0]), Rn[1][0], Rn[1][1], Rn[1][2], float(t[1]),
              Rn[2][0], Rn[2][1], Rn[2][2], float(t[2])]
    return {
        "name": case["name"],
        "model": 1 if "k1_k2" in case else 0,
        "pose12": pose12,
        "X": [float(v) for v in X],
        "z": [float(v) for v in z],
        "intrinsics": [float(fx), float(fy), float(cx), float(cy), float(k1), float(k2), 0.0, 0.0],
        "e": [float(v) for v in e0],
        "jc": [[float(v) for v in row] for row in jc],
        "jp": [[float(v) for v in row] for row in jp],
    }


CASES = [
    {"name": "pinhole_general", "quat_wxyz": (4, 1, 2, 3), "t": ["1/10", "-1/5", "3"],
     "X": ["1/2", "-1/3", "5/4"], "z": ["601/2", "1001/4"], "fx_fy_cx_cy": ["500", "500", "320", "240"]},
    {"name": "pinhole_near", "quat_wxyz": (7, -1, 1, 2), "t": ["-3/2", "1/4", "1"],
     "X": ["-1/8", "2/3", "1/5"], "z": ["100", "400"], "fx_fy_cx_cy": ["458", "457", "367", "248"]},
    {"name": "pinhole_identity", "quat_wxyz": (1, 0, 0, 0), "t": ["0", "0", "0"],
     "X": ["1/4", "-1/8", "2"], "z": ["383", "210"], "fx_fy_cx_cy": ["500", "500", "320", "240"]},
    {"name": "radial", "quat_wxyz": (5, 1, -2, 1), "t": ["1/3", "-1/7", "4"],
     "X": ["-3/4", "1/2", "1"], "z": ["250", "270"], "fx_fy_cx_cy": ["500", "500", "320", "240"],
     "k1_k2": ["-1/10", "1/100"]},
]


def make_known_answer():
    out = [edge_known_answer(c) for c in CASES]
    (HERE / "known_answer.json").write_text(json.dumps(out, indent=1))


def make_ring_fixture():
    from nav24_gb300.synth import Synth, workload_options
    from oracle import oracle
    s = Synth(0)
    p = s.window(0)
    o = workload_options(0)
    r = oracle.solve(p, o, n_threads=1)
    np.savez_compressed(
        HERE / "ring_fixture.npz",
        cam_pose=p.cam_pose, cam_fixed=p.cam_fixed, points=p.points, obs_uv=p.obs_uv, obs_cam=p.obs_cam,
        obs_point=p.obs_point, intrinsics=p.intrinsics,
        out_cam_pose=r.cam_pose, out_points=r.points, out_cost_trace=r.cost_trace,
        out_iterations=np.int32(r.stats["iterations_done"]), out_termination=np.int32(r.stats["termination"]))


SYNTH_CASES = [
    {"family": 0},
    {"family": 1, "n_cams": 40, "n_points": 3000},
    {"family": 2, "n_windows": 8},
    {"family": 3, "n_windows": 4},
    {"family": 4, "n_cams": 60, "n_points": 6000, "seed": 8},
]


def make_synth_digests():
    from nav24_gb300.synth import Synth
    out = [dict(case, digest=Synth(**case).digest()) for case in SYNTH_CASES]
    (HERE / "synth_digests.json").write_text(json.dumps(out, indent=1))


if __name__ == "__main__":
    make_known_answer()
    make_ring_fixture()
    make_synth_digests()
    print("written", sorted(x.name for x in HERE.iterdir()))
