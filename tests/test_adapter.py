"""The C++ drop-in adapter BE::GraphOptimGpu (nav24_gb300/adapter): builds against nav24's data-model
interface (here its header-only stand-ins) and, on a GPU, mutates nav24 objects exactly as
GraphOptim::solve does, with the reference's float roundings (BE_GraphOptim.cpp:147,178,239)."""
import subprocess
from pathlib import Path

import numpy as np
import pytest

from nav24_gb300 import abi
from nav24_gb300.synth import Synth, workload_options

ROOT = Path(__file__).resolve().parent.parent
ADAPTER = ROOT / "nav24_gb300" / "adapter"


def build_roundtrip(out_dir: Path, product_lib: Path) -> Path:
    exe = out_dir / "adapter_roundtrip"
    cmd = ["g++", "-O2", "-std=c++17", "-Wall", "-Wextra", "-I", str(ADAPTER), "-I", str(ADAPTER / "nav24_headers"),
           "-I", str(ROOT / "include"), str(ROOT / "tests" / "adapter" / "adapter_roundtrip.cpp"),
           str(ADAPTER / "GraphOptimGpu.cpp"), "-L", str(product_lib.parent), "-lnavba",
           f"-Wl,-rpath,{product_lib.parent}", "-o", str(exe)]
    subprocess.run(cmd, check=True)
    return exe


def test_adapter_compiles_against_nav24_interface(tmp_path, product_lib):
    assert build_roundtrip(tmp_path, product_lib).exists()


def write_problem(path: Path, p: abi.Problem, iterations: int, robust: int, precision: int, edge_cases: int = 0):
    with open(path, "wb") as f:
        np.array([p.n_cams, p.n_points, p.n_obs, iterations, robust, precision, edge_cases, 0], np.int32).tofile(f)
        p.intrinsics[:4].astype(np.float64).tofile(f)
        p.cam_pose.astype(np.float64).tofile(f)
        p.points.astype(np.float64).tofile(f)
        p.obs_uv.astype(np.float64).tofile(f)
        (p.cam_fixed if p.cam_fixed is not None else np.zeros(p.n_cams)).astype(np.int32).tofile(f)
        (p.point_fixed if p.point_fixed is not None else np.zeros(p.n_points)).astype(np.int32).tofile(f)
        p.obs_cam.astype(np.int32).tofile(f)
        p.obs_point.astype(np.int32).tofile(f)


def read_output(path: Path, p: abi.Problem):
    raw = path.read_bytes()
    st = np.frombuffer(raw[:8], np.int32)
    o = 8
    poses = np.frombuffer(raw[o:o + 8 * 12 * p.n_cams], np.float64).reshape(-1, 12); o += 8 * 12 * p.n_cams
    optids = np.frombuffer(raw[o:o + 8 * p.n_cams], np.uint64); o += 8 * p.n_cams
    pts = np.frombuffer(raw[o:o + 8 * 3 * p.n_points], np.float64).reshape(-1, 3); o += 8 * 3 * p.n_points
    costs = np.frombuffer(raw[o:o + 16], np.float64)
    return st, poses, optids, pts, costs


@pytest.mark.gpu
@pytest.mark.parametrize("robust", [0, 1])
def test_adapter_matches_oracle_with_reference_rounding(tmp_path, product_lib, robust):
    from oracle import oracle
    exe = build_roundtrip(tmp_path, product_lib)
    p = Synth(0).window(0)
    it = 10
    write_problem(tmp_path / "in.bin", p, it, robust, abi.FP64)
    subprocess.run([str(exe), str(tmp_path / "in.bin"), str(tmp_path / "out.bin")], check=True)
    raw = (tmp_path / "out.bin").read_bytes()
    st = np.frombuffer(raw[:8], np.int32)
    o = 8
    poses = np.frombuffer(raw[o:o + 8 * 12 * p.n_cams], np.float64).reshape(-1, 12); o += 8 * 12 * p.n_cams
    optids = np.frombuffer(raw[o:o + 8 * p.n_cams], np.uint64); o += 8 * p.n_cams
    pts = np.frombuffer(raw[o:o + 8 * 3 * p.n_points], np.float64).reshape(-1, 3); o += 8 * 3 * p.n_points
    costs = np.frombuffer(raw[o:o + 16], np.float64)
    assert st[0] == abi.OK
    assert np.all(optids == np.iinfo(np.uint64).max)  # setOptId(-1) on every pose vertex
    # the reference solves the float-rounded problem and writes float-rounded points back
    q = p.copy()
    q.points = q.points.astype(np.float32).astype(np.float64)
    q.obs_uv = q.obs_uv.astype(np.float32).astype(np.float64)
    q.intrinsics = q.intrinsics.astype(np.float32).astype(np.float64)
    opt = abi.default_options(iterations=it, robust=robust)
    r = oracle.solve(q, opt)
    assert abs(costs[1] - r.stats["final_cost"]) / r.stats["final_cost"] < 1e-6
    assert np.array_equal(pts, pts.astype(np.float32).astype(np.float64))
    assert np.allclose(pts, r.points.astype(np.float32), rtol=0, atol=1e-5)
    assert np.allclose(poses, r.cam_pose, rtol=0, atol=1e-7)


def expected_graph(p: abi.Problem):
    """The problem GraphOptim::solve builds from the round trip's edge cases (restated from
    BE_GraphOptim.cpp:79-211 and the patterns in tests/adapter/adapter_roundtrip.cpp): returns
    (problem, camera index of each pose vertex, point index of each point vertex)."""
    no_pose, nov = 3, -1
    k = np.arange(p.n_obs)
    frame = p.obs_cam.astype(np.int64).copy()   # >= 0: a problem frame; -2: frame A; -3: frame B
    frame[k % 17 == 5] = -2
    frame[(k % 17 != 5) & (k % 19 == 7)] = -3
    cams = [c for c in range(p.n_cams) if c != no_pose]   # frames with a pose, id order (:87-90)
    vid = {c: i for i, c in enumerate(cams)}
    opt_id = {**vid, no_pose: nov, -2: 0, -3: nov}          # frame optIds seen by the edges
    valid_obs = (k % 13 != 0) & (p.obs_point % 97 != 3)
    keypoint = k % 11 != 1
    # points in first-seen order over the problem frames' observation lists (:102-115)
    seen = []
    for c in range(p.n_cams):
        for o in np.nonzero(frame == c)[0]:
            if p.obs_point[o] not in seen:
                seen.append(int(p.obs_point[o]))
    pts, uv, oc, op = [], [], [], []
    for i in seen:
        if i % 50 == 7:                                       # invalid point (:143-144)
            continue
        edges = [o for o in np.nonzero(p.obs_point == i)[0]
                 if valid_obs[o] and 0 <= opt_id[int(frame[o])] < len(cams) and keypoint[o]]  # :160-172
        if not edges:                                         # a point without an edge (:204-205)
            continue
        for o in edges:
            uv.append(p.obs_uv[o].astype(np.float32))         # getPointUd is a float
            oc.append(opt_id[int(frame[o])])
            op.append(len(pts))
        pts.append(i)
    q = abi.Problem(cam_pose=p.cam_pose[cams], points=p.points[pts].astype(np.float32).astype(np.float64),
                    obs_uv=np.array(uv, np.float64), obs_cam=oc, obs_point=op,
                    intrinsics=p.intrinsics.astype(np.float32).astype(np.float64),
                    cam_fixed=p.cam_fixed[cams])
    return q, cams, pts


@pytest.mark.gpu
def test_adapter_applies_graph_assembly_filters(tmp_path, product_lib):
    """Invalid observations, observations that are not KeyPoint2D, observations whose frame is
    outside the problem (optId 0: attached to pose vertex 0, as g2o's vertex lookup does; optId -1:
    dropped), a frame without a pose, invalid points and points left without an edge: the adapter
    builds the same graph as GraphOptim and mutates only what GraphOptim would."""
    from oracle import oracle
    exe = build_roundtrip(tmp_path, product_lib)
    p = Synth(0).window(0)
    it = 10
    write_problem(tmp_path / "in.bin", p, it, 1, abi.FP64, edge_cases=1)
    subprocess.run([str(exe), str(tmp_path / "in.bin"), str(tmp_path / "out.bin")], check=True)
    st, poses, optids, pts, costs = read_output(tmp_path / "out.bin", p)
    assert st[0] == abi.OK
    q, cams, kept = expected_graph(p)
    r = oracle.solve(q, abi.default_options(iterations=it, robust=1))
    assert abs(costs[0] - r.stats["initial_cost"]) / r.stats["initial_cost"] < 1e-12
    assert abs(costs[1] - r.stats["final_cost"]) / r.stats["final_cost"] < 1e-6
    # pose vertices: new poses, optId -1; the frame without a pose is untouched (optId stays -1)
    assert np.allclose(poses[cams], r.cam_pose, rtol=0, atol=1e-7)
    assert np.all(np.isnan(poses[3])) and optids[3] == np.iinfo(np.uint64).max
    assert np.all(optids[cams] == np.iinfo(np.uint64).max)
    # point vertices get float-rounded solutions; every other point keeps its input position
    assert np.allclose(pts[kept], r.points.astype(np.float32), rtol=0, atol=1e-5)
    others = np.setdiff1d(np.arange(p.n_points), kept)
    assert others.size > 0 and np.array_equal(pts[others], p.points[others])
