"""Benchmark of the GB300 bundle-adjustment back end.

Workload (default, `--workload windows`): batched local BA, 512 independent windows
(5-20 keyframes, 200-3000 points, 3-8 views per point, 0.8 px noise, first two keyframes fixed,
10 LM iterations each), seeded synthetic data (family 2, seed 1002).  One step = one solve of
the whole batch from its initial state (one persistent kernel launch).

Metric: BA observations/s = sum over windows of active edges x LM iterations completed, per
second of solve; reported for the mixed form (`value`) beside the plain FP64 form, with the
LM iterations/s of both and the final-cost agreement of the two forms.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

`--impl reference` times nav24's BA algorithm on the host cores instead: the reference's own g2o
path cannot be built here (g2o, Eigen, OpenCV are absent), so the CPU restatement of it
(oracle/, FP64, one window per thread, all host threads) runs the same workload.

The line also carries, under "workloads", one solve of each other named workload on the same GPU
(after one warm-up solve): the 200-camera grid (mixed vs FP64), the differentiable sphere cap
(forward and backward through K = 5 LM steps) and the large robust figure-eight with shared
distortion (PCG, mixed vs FP64).  `--no-secondary` skips them.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

import numpy as np  # noqa: E402

METRIC = "BA obs/s (resid+Jac+Schur) & LM iter/s: mixed vs FP64 GPU at same final cost"
UNIT = "obs/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=["windows"], default="windows")
    ap.add_argument("--windows", type=int, default=512)
    ap.add_argument("--cpu-sample", type=int, default=512, help="windows in the CPU baseline sample")
    ap.add_argument("--profile-case", choices=["mixed", "fp64", "grid", "pcg", "vjp", "pose", "twoview", "undistort",
                                               "kb8"],
                    default=None,
                    help="run only the device-resident solves of one precision (mixed, fp64), or one solve of a "
                         "secondary workload (for profiler captures)")
    ap.add_argument("--no-secondary", action="store_true", help="skip the secondary workloads")
    ap.add_argument("--pcg-cams", type=int, default=1000, help="cameras of the figure-eight PCG workload")
    ap.add_argument("--profile-precision", choices=["both", "fp64", "mixed"], default="both",
                    help="precisions the grid and PCG profile cases run")
    ap.add_argument("--pcg-points", type=int, default=500000, help="points of the figure-eight PCG workload")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class Dist:
    """Barrier and max/sum over ranks (one process per GPU, replicas only: nothing on the data path);
    no-ops for one rank.  Backend "nccl" (GPU tensors) on the GPU nodes, "gloo" (CPU tensors) for
    host-only runs."""

    def __init__(self, world: int, local: int, backend: str = "nccl"):
        self.world = world
        self.backend = backend
        if world > 1:
            import torch
            import torch.distributed as td
            if backend == "nccl":
                torch.cuda.set_device(local)
            td.init_process_group(backend)
            self.td, self.torch = td, torch

    def barrier(self):
        if self.world > 1:
            self.td.barrier()

    def _reduce(self, x: float, op) -> float:
        t = self.torch.tensor([x], dtype=self.torch.float64, device="cuda" if self.backend == "nccl" else "cpu")
        self.td.all_reduce(t, op=op)
        return float(t.item())

    def max(self, x: float) -> float:
        return x if self.world == 1 else self._reduce(x, self.td.ReduceOp.MAX)

    def sum(self, x: float) -> float:
        return x if self.world == 1 else self._reduce(x, self.td.ReduceOp.SUM)

    def close(self):
        if self.world > 1:
            self.td.destroy_process_group()


def replica_seed(rank: int) -> int:
    """Each rank solves its own 512 windows (weak scaling): family 2, seed 1002 + 7919 rank."""
    return 1002 + 7919 * rank


def whole_job_rate(dist: Dist, work: float, seconds: float) -> float:
    """Whole-job throughput over replicas: the work of every rank over the slowest rank's time."""
    return dist.sum(work) / dist.max(seconds)


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms while running."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except FileNotFoundError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        sm = [float(r[1]) for r in self.rows if len(r) > 8 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) > 8 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows if len(r) > 8 for i in range(4) if r[5 + i] == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def algorithmic_bytes(wins, results, s_o: int, s_d: int = 8) -> float:
    """Algorithmic DRAM bytes of one batched solve (per-window sums of the per-iteration model:
    linearize+reduce, Schur assembly, back-substitution+update, trial cost per damping trial)."""
    total = 0.0
    for w, r in zip(wins, results):
        st = r.stats
        No, Np, Nc = st["n_active_edges"], st["n_free_points"], st["n_free_cams"]
        it = st["iterations_done"]
        trials = st["trials_accepted"] + st["trials_rejected"]
        nnz = st["n_schur_blocks"]
        lin = No * (2 * s_o + 8) + Np * 3 * s_o + Nc * 7 * s_d + Np * 9 * s_o + Nc * 27 * s_o
        schur = No * (2 * s_o + 8) + Np * 9 * s_o + nnz * 36 * s_d + Nc * 6 * s_d
        upd = No * (2 * s_o + 8) + Np * (3 * s_o * 2 + 9 * s_o) + Nc * (6 + 7 * 2) * s_d
        cost = No * (2 * s_o + 8) + Np * 3 * s_o + Nc * 7 * s_d
        total += it * lin + trials * (schur + upd + cost) + cost
    return total


def profile_traffic():
    """DRAM traffic per launch from the committed ncu summary, if one exists."""
    p = ROOT / "profiles" / "window_lm_kernel_traffic.json"
    if p.exists():
        return json.loads(p.read_text())
    return None


def fp64_roofline():
    """The plain FP64 window kernel's bound: its FP64 pipe, from the committed ncu summary
    (sm__pipe_fp64_cycles_active of one launch), beside its DRAM throughput; None without one."""
    p = ROOT / "profiles" / "window_lm_kernel_fp64_pipe.json"
    if not p.exists():
        return None
    d = json.loads(p.read_text())
    return {"bound": "fp64", "kernel": "window_lm_kernel<double>", "achieved": d["fp64_pipe_active_pct"],
            "peak": 100.0, "unit": "% of FP64 pipe cycles", "frac": d["fp64_pipe_active_pct"] / 100.0,
            "dram_frac_of_peak": d.get("dram_throughput_pct"), "source": d.get("captured")}


def cpu_reference(wins, opt, n_threads):
    from oracle import oracle
    t0 = time.perf_counter()
    with ThreadPoolExecutor(n_threads) as ex:
        res = list(ex.map(lambda w: oracle.solve(w, opt, n_threads=1), wins))
    dt = time.perf_counter() - t0
    edge_it = sum(r.stats["n_active_edges"] * r.stats["iterations_done"] for r in res)
    iters = sum(r.stats["iterations_done"] for r in res)
    return dt, edge_it, iters, res


def run_reference(args, rank, world):
    from nav24_gb300.synth import Synth, workload_options
    from nav24_gb300 import abi
    if rank != 0:
        return
    s = Synth(2, n_windows=args.windows)
    wins = s.windows()[: args.cpu_sample]
    opt = workload_options(2, abi.FP64)
    nth = os.cpu_count() or 1
    for _ in range(args.warmup):
        cpu_reference(wins[: max(1, len(wins) // 8)], opt, nth)
    times, eis, its = [], 0, 0
    for _ in range(args.steps):
        dt, ei, it, _ = cpu_reference(wins, opt, nth)
        times.append(dt)
        eis, its = ei, it
    t = float(np.mean(times))
    val = eis / t
    line = {
        "impl": "reference", "metric": METRIC, "value": val, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": t * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"batched local BA, {len(wins)} windows of family 2 (seed 1002), FP64 CPU "
                               f"restatement of nav24 GraphOptim + g2o LM", "windows": len(wins),
                   "lm_iterations": 10},
        "lm_iter_per_s": its / t,
        "cpu_baseline": {"value": val, "unit": UNIT, "cores": nth, "kind": "port",
                         "sample": f"{len(wins)} windows x 10 LM iterations, one window per thread"},
        "e2e": {"value": val, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def time_device(ctx, wins, opt, steps, warmup, dist):
    """Device-resident solves: prepare once, then `steps` launches timed with CUDA events."""
    ctx.prepare_batched(wins, opt)
    for _ in range(warmup):
        ctx.run(opt)
    dist.barrier()
    ms, stats = [], None
    for _ in range(steps):
        stats = ctx.run(opt)
        ms.append(stats["time_solve_ms"])
    dist.barrier()
    results = ctx.fetch_batched(opt)
    return ms, stats, results


def solve_pair(ctx, p, family, precisions=("fp64", "mixed")):
    """One warm-up and one timed solve of problem p in each precision; device time per solve."""
    from nav24_gb300 import abi
    from nav24_gb300.synth import workload_options
    out = {}
    for name, prec in (("fp64", abi.FP64), ("mixed", abi.MIXED)):
        if name not in precisions:
            continue
        o = workload_options(family, prec)
        ctx.solve(p, o)
        r = ctx.solve(p, o)
        t = r.stats["time_solve_ms"] * 1e-3
        out[name] = {"obs_per_s": r.stats["edge_iterations"] / t, "lm_iter_per_s": r.stats["iterations_done"] / t,
                     "ms": t * 1e3, "final_cost": r.stats["final_cost"], "initial_cost": r.stats["initial_cost"],
                     "iterations": r.stats["iterations_done"], "pcg_iterations": r.stats["pcg_iterations_total"]}
    if len(out) == 2:
        out["mixed_over_fp64"] = out["mixed"]["obs_per_s"] / out["fp64"]["obs_per_s"]
        out["final_cost_rel_diff"] = abs(out["mixed"]["final_cost"] - out["fp64"]["final_cost"]) / out["fp64"]["final_cost"]
    return out


def twoview_workload(ctx):
    """nav_ba_twoview_check on synthetic matches: one frame pair at a typical match count, and a
    large batch of matches for throughput."""
    K = np.array([500.0, 500.0, 320.0, 240.0])
    res = {}
    for n in (2000, 1 << 18):
        rng = np.random.default_rng(1006)
        rv = np.array([0.02, -0.06, 0.01])
        th = np.linalg.norm(rv)
        kx = np.array([[0, -rv[2], rv[1]], [rv[2], 0, -rv[0]], [-rv[1], rv[0], 0]]) / th
        R = np.eye(3) + np.sin(th) * kx + (1 - np.cos(th)) * kx @ kx
        t = np.array([-0.3, 0.02, 0.01])
        X = np.stack([rng.uniform(-2, 2, n), rng.uniform(-1.5, 1.5, n), rng.uniform(2, 8, n)], axis=1)
        proj = lambda P: np.stack([K[0] * P[:, 0] / P[:, 2] + K[2], K[1] * P[:, 1] / P[:, 2] + K[3]], axis=1)
        kp1 = proj(X) + 0.5 * rng.standard_normal((n, 2))
        kp2 = proj(X @ R.T + t) + 0.5 * rng.standard_normal((n, 2))
        bad = rng.random(n) < 0.1
        kp2[bad] = np.stack([rng.uniform(0, 640, bad.sum()), rng.uniform(0, 480, bad.sum())], axis=1)
        u = t / np.linalg.norm(t)
        ux = np.array([[0, -u[2], u[1]], [u[2], 0, -u[0]], [-u[1], u[0], 0]])
        tw = np.eye(3) + 2 * ux @ ux  # rotation by pi about t
        Rs = np.stack([R, R, tw @ R, tw @ R])
        ts_ = np.stack([t, -t, t, -t])
        th2 = 4.0  # 4 sigma^2 with sigma = 1 px, as the reconstruction's CheckRT calls it
        ctx.twoview_check(K, kp1, kp2, Rs, ts_, th2, 0.99998)
        ts = []
        for _ in range(5):
            t0 = time.perf_counter()
            r = ctx.twoview_check(K, kp1, kp2, Rs, ts_, th2, 0.99998)
            ts.append(time.perf_counter() - t0)
        dt = float(np.median(ts))
        res[f"{n}_matches"] = {"hypotheses": 4, "matches": n, "ms": dt * 1e3, "checks_per_s": 4 * n / dt,
                               "n_good": [int(v) for v in r["n_good"]]}
    res["workload"] = ("4 relative-pose hypotheses x matches of one frame pair (0.3 m baseline, points 2-8 m, "
                       "0.5 px noise, 10% outliers); per match: linear triangulation (4x4 SVD), cheirality, "
                       "reprojection gates, parallax")
    res["timing"] = "median wall clock of 5 C-ABI calls with host buffers (copies in, kernel, copies out)"
    return res


KB8_INTR = np.array([380.0, 380.0, 320.0, 240.0, -0.012, 0.0025, -0.0006, 0.00008])


def kb8_windows(n_windows, seed=1002, noise=1.0):
    """The batched-window family's windows with their observations made through the Kannala-Brandt
    fisheye model (theta = atan2(rho, z), r = theta + k1 theta^3 + ... + k4 theta^9) from the true
    geometry, 1 px noise; the pinhole originals alongside."""
    from nav24_gb300 import abi
    from nav24_gb300.synth import Synth
    s = Synth(2, seed=seed, n_windows=n_windows)
    rng = np.random.default_rng(seed + 5)
    kb, ph = [], []
    k = KB8_INTR
    for w in range(n_windows):
        truth, init = s.window(w, truth=True), s.window(w)
        P = truth.cam_pose.reshape(-1, 3, 4)
        Xc = np.einsum("nij,nj->ni", P[truth.obs_cam, :, :3], truth.points[truth.obs_point]) + P[truth.obs_cam, :, 3]
        th = np.arctan2(np.hypot(Xc[:, 0], Xc[:, 1]), Xc[:, 2])
        psi = np.arctan2(Xc[:, 1], Xc[:, 0])
        r = th + k[4] * th ** 3 + k[5] * th ** 5 + k[6] * th ** 7 + k[7] * th ** 9
        uv = np.stack([k[0] * r * np.cos(psi) + k[2], k[1] * r * np.sin(psi) + k[3]], axis=1)
        q = init.copy()
        q.obs_uv = np.ascontiguousarray(uv + noise * rng.standard_normal(uv.shape))
        q.intrinsics = k.copy()
        q.camera_model = abi.CAM_KANNALA_BRANDT8
        kb.append(q)
        ph.append(init)
    return kb, ph


def kb8_workload(ctx, n_windows=128):
    from nav24_gb300 import abi
    from nav24_gb300.synth import workload_options
    kb, ph = kb8_windows(n_windows)
    res = {"workload": f"{n_windows} windows of the batched family observed through the Kannala-Brandt 8 "
                       "model (1 px noise), 10 LM iterations, one batched call; the same windows with "
                       "their pinhole observations alongside",
           "timing": "median wall clock of 3 nav_ba_solve_batched calls with host buffers; device_ms = "
                     "the calls' time_solve_ms"}
    for model, probs in (("kb8", kb), ("pinhole", ph)):
        for name, prec in (("fp64", abi.FP64), ("mixed", abi.MIXED)):
            o = workload_options(2, prec)
            ctx.solve_batched(probs, o)
            ts, rr = [], None
            for _ in range(3):
                t0 = time.perf_counter()
                rr = ctx.solve_batched(probs, o)
                ts.append(time.perf_counter() - t0)
            dt = float(np.median(ts))
            ei = sum(r.stats["edge_iterations"] for r in rr)
            res[f"{model}_{name}"] = {"ms": dt * 1e3, "obs_per_s": ei / dt, "device_ms": rr[0].stats["time_solve_ms"],
                                      "final_cost_sum": float(sum(r.stats["final_cost"] for r in rr)),
                                      "status_ok": int(sum(r.status == abi.OK for r in rr))}
    return res


def secondary_workloads(ctx, only=None, pcg_cams=1000, pcg_points=500000, precisions=("fp64", "mixed")):
    """One solve of each other named workload (device time, including the per-solve upload)."""
    from nav24_gb300 import abi
    from nav24_gb300.synth import Synth, workload_options
    out = {}
    if only in (None, "grid"):
        p = Synth(1).window(0)
        out["grid_200cams"] = {"workload": "200 cameras on a 20x10 grid facing down, 50,000 points, Huber 2 px, "
                                           "20 LM iterations (family 1, seed 1001), grid engine, Cholesky",
                               "observations": p.n_obs, **solve_pair(ctx, p, 1, precisions)}
    if only in (None, "vjp"):
        p = Synth(3).window(0)
        o = workload_options(3)
        ctx.vjp(p, o)
        t0 = time.perf_counter()
        r, lam, _ = ctx.vjp(p, o)
        t1 = time.perf_counter()
        _, _, g = ctx.vjp(p, o, lam, cost_bar=1.0)
        t2 = time.perf_counter()
        out["differentiable_cap"] = {
            "workload": "50 cameras on a sphere cap, 10,000 points, Huber 2 px, K = 5 LM iterations (family 3, "
                        "seed 1003); VJP w.r.t. observations and intrinsics", "observations": p.n_obs,
            "forward_ms": (t1 - t0) * 1e3, "replay_and_backward_ms": (t2 - t1) * 1e3, "steps": len(lam),
            "forward_obs_per_s": r.stats["edge_iterations"] / (t1 - t0), "final_cost": r.stats["final_cost"],
            "timing": "wall clock of the C-ABI call (host graph build, upload, device work, download)"}
    if only in (None, "pose"):
        probs = Synth(2, n_windows=2048, seed=1102).pose_problems()
        o = workload_options(2, abi.MIXED)
        nobs = sum(p.obs_uv.shape[0] for p in probs)
        call = ctx.pose_call(probs, o)  # C structs and output buffers built once: the C ABI is timed
        call()
        ts = []
        for _ in range(5):
            t0 = time.perf_counter()
            call()
            ts.append(time.perf_counter() - t0)
        dt = float(np.median(ts))
        res = call.results()
        its = sum(st["iterations_done"] for _, st in res)
        # one frame per call, as tracking calls it at camera rate
        one = ctx.pose_call([probs[0]], o)
        one()
        t1s = []
        for _ in range(200):
            t1 = time.perf_counter()
            one()
            t1s.append(time.perf_counter() - t1)
        out["tracking_pose_only"] = {
            "workload": "2048 motion-only problems (the last keyframe of each family-2 window against its fixed "
                        "points), 10 LM iterations, mixed form, one launch", "problems": len(probs),
            "observations": nobs, "ms": dt * 1e3, "frames_per_s": len(probs) / dt,
            "obs_per_s": sum(p.obs_uv.shape[0] * st["iterations_done"] for p, (_, st) in zip(probs, res)) / dt,
            "lm_iterations": its, "single_frame_ms": float(np.median(t1s)) * 1e3,
            "single_frame_obs": int(probs[0].obs_uv.shape[0]),
            "timing": "median wall clock of 5 C-ABI calls with host buffers (validation, host layout, upload, "
                      "kernel, download); single_frame_ms: median of 200 calls with one problem"}
    if only in (None, "undistort"):
        # keypoints over a VGA image with a typical radial-tangential calibration, 5 fixed-point
        # iterations (cv::undistortPoints' default count as nav24 calls it)
        K = np.array([458.654, 457.296, 367.215, 248.375])
        D = np.array([-0.28340811, 0.07395907, 0.00019359, 1.76187114e-05])
        rng = np.random.default_rng(1005)
        n = 1 << 21
        uv = np.stack([rng.uniform(0, 752, n), rng.uniform(0, 480, n)], axis=1)
        ctx.undistort_points(K, D, uv[:4096])
        ts = []
        for _ in range(5):
            t0 = time.perf_counter()
            ctx.undistort_points(K, D, uv)
            ts.append(time.perf_counter() - t0)
        dt = float(np.median(ts))
        out["undistort_keypoints"] = {
            "workload": f"{n} keypoints uniform over a 752x480 image, radial-tangential (k1, k2, p1, p2), 5 "
                        "iterations, FP64", "keypoints": n, "ms": dt * 1e3, "keypoints_per_s": n / dt,
            "h2d_bytes": 16 * n, "d2h_bytes": 16 * n,
            "timing": "median wall clock of 5 C-ABI calls with host buffers (copies in, kernel, copies out)"}
    if only in (None, "kb8"):
        out["kb8_windows"] = kb8_workload(ctx)
    if only in (None, "twoview"):
        # map-initialization triangulation: 4 relative-pose hypotheses x matches of one frame pair,
        # points 2-8 m ahead of a 0.3 m baseline, 0.5 px noise, 10% outlier matches
        out["twoview_triangulation"] = twoview_workload(ctx)
    if only in (None, "pcg"):
        p = Synth(4, n_cams=pcg_cams, n_points=pcg_points).window(0)
        out["figure_eight_pcg"] = {
            "workload": f"{pcg_cams} cameras on a {2 * pcg_cams} m figure-eight, {pcg_points} points, shared radial "
                        "k1/k2 optimized, 5% outliers, Huber 1.5 px, 30 LM iterations, PCG (block-Jacobi, tol 1e-6, "
                        "<= 100 iterations) (family 4, seed 1004), grid engine", "observations": p.n_obs,
            **solve_pair(ctx, p, 4, precisions)}
    return out


def main():
    args = parse()
    rank, world, local = dist_env()
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    dist = Dist(world, local)
    from nav24_gb300 import Context, abi
    from nav24_gb300.build import build_all
    from nav24_gb300.synth import Synth, workload_options
    build_all()
    s = Synth(2, seed=replica_seed(rank), n_windows=args.windows)
    wins = s.windows()
    n_obs = s.n_obs
    ctx = Context(local if world > 1 else 0)
    om = workload_options(2, abi.MIXED)
    of = workload_options(2, abi.FP64)

    if args.profile_case in ("grid", "pcg", "vjp", "pose", "twoview", "undistort", "kb8"):
        precs = ("fp64", "mixed") if args.profile_precision == "both" else (args.profile_precision,)
        print(json.dumps(secondary_workloads(ctx, args.profile_case, args.pcg_cams, args.pcg_points, precs)), flush=True)
        ctx.close()
        dist.close()
        return
    if args.profile_case:
        o = om if args.profile_case == "mixed" else of
        ms, st, _ = time_device(ctx, wins, o, args.steps, args.warmup, dist)
        print(json.dumps({"profile_case": args.profile_case, "windows": len(wins), "observations": n_obs,
                          "ms": ms, "edge_iterations": st["edge_iterations"]}), flush=True)
        ctx.close()
        dist.close()
        return
    with ClockSampler(local) as clk:
        ms_m, st_m, res_m = time_device(ctx, wins, om, args.steps, args.warmup, dist)
    clocks = clk.summary()
    ms_f, st_f, res_f = time_device(ctx, wins, of, args.steps, args.warmup, dist)

    t_m = dist.max(float(np.mean(ms_m)) * 1e-3)
    t_f = dist.max(float(np.mean(ms_f)) * 1e-3)
    it_m = dist.sum(float(st_m["iterations_done"]))
    it_f = dist.sum(float(st_f["iterations_done"]))
    value = whole_job_rate(dist, float(st_m["edge_iterations"]), float(np.mean(ms_m)) * 1e-3)
    fp64_value = whole_job_rate(dist, float(st_f["edge_iterations"]), float(np.mean(ms_f)) * 1e-3)
    cost_rel = max(abs(a.stats["final_cost"] - b.stats["final_cost"]) / b.stats["final_cost"]
                   for a, b in zip(res_m, res_f) if b.stats["final_cost"] > 0)

    # end to end through the C ABI with host buffers: every step validates and builds the graph
    # on the host, copies the inputs to the device, solves, and copies the results back
    call = ctx.batched_call(wins, om)
    for _ in range(args.warmup):
        call()
    dist.barrier()
    e2e_t, e2e_ei, h2d, d2h = [], 0, 0, 0
    for _ in range(args.steps):
        t0 = time.perf_counter()
        call()
        e2e_t.append(time.perf_counter() - t0)
    rr = call.results()
    e2e_ei = sum(r.stats["edge_iterations"] for r in rr)
    h2d, d2h = rr[0].stats["h2d_bytes"], rr[0].stats["d2h_bytes"]
    e2e_split = {"host_setup_and_upload_ms": rr[0].stats["time_setup_ms"], "device_ms": rr[0].stats["time_solve_ms"],
                 "download_ms": rr[0].stats["time_download_ms"]}
    dist.barrier()
    e2e_time = dist.max(float(np.mean(e2e_t)))
    e2e_value = dist.sum(float(e2e_ei)) / e2e_time

    # the same end-to-end call in the plain FP64 form (what compares with the FP64 CPU reference
    # arm at the same precision)
    call64 = ctx.batched_call(wins, of)
    for _ in range(args.warmup):
        call64()
    dist.barrier()
    e64_t = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        call64()
        e64_t.append(time.perf_counter() - t0)
    rr64 = call64.results()
    dist.barrier()
    e64_time = dist.max(float(np.mean(e64_t)))
    e64_value = dist.sum(float(sum(r.stats["edge_iterations"] for r in rr64))) / e64_time
    e2e_fp64 = {"value": e64_value, "unit": UNIT, "h2d_bytes_per_step": int(rr64[0].stats["h2d_bytes"]),
                "d2h_bytes_per_step": int(rr64[0].stats["d2h_bytes"]), "ms_per_step": e64_time * 1e3}

    # roofline of the one kernel (window_lm_kernel): algorithmic bytes / launch time
    peak, peak_kind = measured_peaks()
    alg = algorithmic_bytes(wins, res_m, s_o=4)
    achieved = alg / (float(np.mean(ms_m)) * 1e-3) / 1e9
    prof = profile_traffic()
    roofline = {"bound": "hbm", "kernel": "window_lm_kernel<float>", "achieved": achieved, "peak": peak,
                "unit": "GB/s", "frac": achieved / peak, "peak_kind": f"{peak_kind} hbm_gbs",
                "algorithmic_bytes_per_launch": alg,
                "traffic": prof["dram_bytes_per_launch_full"] if prof else None}

    # CPU baseline: the FP64 restatement on this host, all threads, bounded sample
    cpu = None
    oracle_diff = None
    if rank == 0:
        nth = os.cpu_count() or 1
        sample = wins[: args.cpu_sample]
        dt, ei, its, res_o = cpu_reference(sample, of, nth)
        cpu = {"value": ei / dt, "unit": UNIT, "cores": nth, "kind": "port",
               "sample": f"{len(sample)} windows x 10 LM iterations (FP64 oracle), one window per thread"}
        # and on one core, as g2o runs by default (a smaller sample of the same windows)
        one = sample[: max(1, len(sample) // 16)]
        dt1, ei1, _, _ = cpu_reference(one, of, 1)
        cpu["single_thread"] = {"value": ei1 / dt1, "unit": UNIT, "cores": 1,
                                "sample": f"{len(one)} windows x 10 LM iterations (FP64 oracle)"}
        # "same final cost": both GPU forms against the FP64 oracle, per window
        oracle_diff = {
            name: max(abs(a.stats["final_cost"] - b.stats["final_cost"]) / b.stats["final_cost"]
                      for a, b in zip(res, res_o) if b.stats["final_cost"] > 0)
            for name, res in (("mixed", res_m), ("fp64", res_f))}

    secondary = None
    if rank == 0 and not args.no_secondary:
        secondary = secondary_workloads(ctx, None, args.pcg_cams, args.pcg_points)

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_m * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32 bulk / f64 Cholesky+cost+SE3", "data": "synthetic",
            "config": {"workload": "batched local BA: 512 windows (5-20 keyframes, 200-3000 points, "
                                   "3-8 views/point, first two keyframes fixed), 10 LM iterations, "
                                   "family 2 seed 1002 (+7919*rank)",
                       "windows_per_gpu": len(wins), "observations_per_gpu": n_obs,
                       "l2": "inputs+scratch > L2 (no flush needed)", "precision": "mixed",
                       "parallelism": f"replicas x{world}"},
            "lm_iter_per_s": it_m / t_m,
            "fp64": {"value": fp64_value, "unit": UNIT, "ms_per_step": t_f * 1e3, "lm_iter_per_s": it_f / t_f,
                     "e2e": e2e_fp64, "roofline": fp64_roofline()},
            "mixed_over_fp64": value / fp64_value,
            "final_cost_rel_diff_max": cost_rel,
            "final_cost_rel_diff_vs_oracle_max": oracle_diff,
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h), "ms_per_step": e2e_time * 1e3, "last_call": e2e_split},
            "roofline": roofline,
            "cpu_baseline": cpu,
            "clocks": clocks,
            "gpu_launches": args.steps,
            "workloads": secondary,
        }
        print(json.dumps(line), flush=True)
    ctx.close()
    dist.close()


if __name__ == "__main__":
    main()
