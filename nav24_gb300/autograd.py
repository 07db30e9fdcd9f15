"""torch.autograd.Function over nav_ba_vjp: bundle adjustment as a differentiable layer.

    cost, poses, points = bundle_adjust(obs_uv, intrinsics, problem, options)

runs K LM iterations (options.iterations) of the problem with its observations and pinhole
intrinsics (fx, fy, cx, cy) taken from the two tensors, and returns the final robust cost, the
optimized poses [n_cams, 12] and points [n_points, 3] as FP64 tensors on obs_uv's device.  The
backward differentiates the solve with its damping schedule frozen (the accepted steps of the
forward, each at its damping; nav_ba_vjp in include/nav_ba.h) with respect to obs_uv (float32 or
float64; the gradient comes back in the input's dtype) and the intrinsics.  Jacobians are
recomputed on the GPU in the backward, not stored.  The forward keeps only the schedule.

The library computes on the GPU through the C ABI with host buffers, so tensors are staged through
host memory; torch is imported only here.
"""
from __future__ import annotations

import numpy as np
import torch

from . import abi
from ._lib import Context


def _problem_with(problem: abi.Problem, uv: np.ndarray, k4: np.ndarray) -> abi.Problem:
    p = problem.copy()
    p.obs_uv = np.ascontiguousarray(uv, np.float64).reshape(-1, 2)
    intr = p.intrinsics.copy()
    intr[:4] = k4
    p.intrinsics = intr
    return p


class BundleAdjust(torch.autograd.Function):
    @staticmethod
    def forward(fctx, obs_uv: torch.Tensor, intrinsics: torch.Tensor, problem: abi.Problem,
                options: abi.nav_ba_options, context: Context):
        uv = obs_uv.detach().to("cpu", torch.float64).numpy()
        k4 = intrinsics.detach().to("cpu", torch.float64).numpy().reshape(4)
        p = _problem_with(problem, uv, k4)
        res, lambdas, _ = context.vjp(p, options)
        fctx.state = (p, options, context, lambdas, obs_uv.dtype, intrinsics.dtype)
        dev = obs_uv.device
        cost = torch.tensor(res.stats["final_cost"], dtype=torch.float64, device=dev)
        poses = torch.from_numpy(res.cam_pose.copy()).to(dev)
        points = torch.from_numpy(res.points.copy()).to(dev)
        return cost, poses, points

    @staticmethod
    def backward(fctx, g_cost, g_poses, g_points):
        p, options, context, lambdas, uv_dtype, k_dtype = fctx.state
        cb = 0.0 if g_cost is None else float(g_cost.detach().to("cpu", torch.float64))
        pb = None if g_poses is None else g_poses.detach().to("cpu", torch.float64).numpy()
        xb = None if g_points is None else g_points.detach().to("cpu", torch.float64).numpy()
        _, _, g = context.vjp(p, options, lambdas, cost_bar=cb, pose_bar=pb, point_bar=xb)
        dev = g_cost.device if g_cost is not None else "cpu"
        g_uv = torch.from_numpy(g["obs_uv"]).to(dev, uv_dtype)
        g_k = torch.from_numpy(g["intrinsics"]).to(dev, k_dtype)
        return g_uv, g_k, None, None, None


def bundle_adjust(obs_uv: torch.Tensor, intrinsics: torch.Tensor, problem: abi.Problem,
                  options: abi.nav_ba_options, context: Context):
    """Differentiable BA; see the module docstring."""
    return BundleAdjust.apply(obs_uv, intrinsics, problem, options, context)
