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


def write_problem(path: Path, p: abi.Problem, iterations: int, robust: int, precision: int):
    with open(path, "wb") as f:
        np.array([p.n_cams, p.n_points, p.n_obs, iterations, robust, precision, 0, 0], np.int32).tofile(f)
        p.intrinsics[:4].astype(np.float64).tofile(f)
        p.cam_pose.astype(np.float64).tofile(f)
        p.points.astype(np.float64).tofile(f)
        p.obs_uv.astype(np.float64).tofile(f)
        (p.cam_fixed if p.cam_fixed is not None else np.zeros(p.n_cams)).astype(np.int32).tofile(f)
        (p.point_fixed if p.point_fixed is not None else np.zeros(p.n_points)).astype(np.int32).tofile(f)
        p.obs_cam.astype(np.int32).tofile(f)
        p.obs_point.astype(np.int32).tofile(f)


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
