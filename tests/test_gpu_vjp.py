"""GPU tests of the differentiable solve (nav_ba_vjp) on the sphere-cap workload (family 3: 50
cameras on a sphere cap, 10,000 points, about 6 views per point, Huber 2 px, K = 5 LM iterations).

The differentiated function is the solve with its damping schedule frozen (the accepted steps,
each at its recorded damping).  Checks:
  - the recorded forward equals nav_ba_solve's result, the GPU replay reproduces it exactly, and
    the oracle records the same schedule and replays it to the same outputs;
  - at K = 0 the backward of the cost is the reference's Jacobian-derived gradient 2 J^T W e
    (the oracle's linearization, EdgeSE3ProjectXYZ::linearizeOplus) in every block;
  - the VJP against a random unit-norm upstream gradient matches FP64 central differences
    (step 1e-6) of the replay on 200 random coordinates (all four intrinsics and 196 observation
    coordinates) within 1e-5 relative, both for the GPU replay and for the oracle's replay, as a
    vector norm; and coordinate by coordinate against fourth-order central differences (step
    1e-4, less rounding noise), each within 1e-5 of max(|fd_k|, 1% of the largest);
  - the torch.autograd.Function returns the same gradients, in float32 for float32 observations.
"""
import numpy as np
import pytest

from nav24_gb300 import abi
from nav24_gb300.synth import Synth, workload_options
from oracle import oracle

pytestmark = pytest.mark.gpu


def rel(a, b):
    return abs(a - b) / abs(b)


def vrel(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b))


def small():
    return Synth(3, n_cams=16, n_points=1500, seed=11).window(0)


def upstream(p, seed):
    rng = np.random.default_rng(seed)
    v = rng.standard_normal(1 + 12 * p.n_cams + 3 * p.n_points)
    v /= np.linalg.norm(v)
    return v[0], v[1:1 + 12 * p.n_cams].reshape(-1, 12), v[1 + 12 * p.n_cams:].reshape(-1, 3)


def loss(r, cb, pb, xb):
    return cb * r.stats["final_cost"] + float(np.sum(pb * r.cam_pose)) + float(np.sum(xb * r.points))


def with_theta(p, k, val):
    """Problem with coordinate k of theta = (fx, fy, cx, cy, obs_uv.ravel()) set to val."""
    q = p.copy()
    if k < 4:
        q.intrinsics[k] = val
    else:
        q.obs_uv.reshape(-1)[k - 4] = val
    return q


def theta_of(p, k):
    return p.intrinsics[k] if k < 4 else p.obs_uv.reshape(-1)[k - 4]


def grad_of(g, k):
    return g["intrinsics"][k] if k < 4 else g["obs_uv"].reshape(-1)[k - 4]


def coords(p, n, seed):
    rng = np.random.default_rng(seed)
    return [0, 1, 2, 3] + list(4 + rng.choice(2 * p.n_obs, n - 4, replace=False))


def test_record_and_replay(ctx):
    p = small()
    o = workload_options(3)
    r, lam, _ = ctx.vjp(p, o)
    s = ctx.solve(p, o)
    assert r.status == abi.OK and 1 <= len(lam) == r.stats["trials_accepted"]
    assert rel(r.stats["final_cost"], s.stats["final_cost"]) < 1e-10
    assert np.max(np.abs(r.points - s.points)) < 1e-9
    r2, _, _ = ctx.vjp(p, o, lam)
    assert r2.stats["final_cost"] == r.stats["final_cost"]
    assert np.array_equal(r2.cam_pose, r.cam_pose) and np.array_equal(r2.points, r.points)
    ro, lam_o = oracle.solve_schedule(p, o, n_threads=8)
    assert len(lam_o) == len(lam) and np.allclose(lam_o, lam, rtol=1e-8)
    ro2, _ = oracle.solve_schedule(p, o, lam, n_threads=8)
    assert rel(ro2.stats["final_cost"], r.stats["final_cost"]) < 1e-10
    assert np.max(np.abs(ro2.cam_pose - r.cam_pose)) < 1e-9
    assert np.max(np.abs(ro2.points - r.points)) < 1e-9


def test_zero_steps_gives_jacobian_gradient(ctx):
    """d cost / d (pose, point, z, K) at the initial state = 2 sum w J^T e (oracle linearization)."""
    p = small()
    o = workload_options(3)
    _, _, g = ctx.vjp(p, o, [], cost_bar=1.0)
    e, jc, jp, w = oracle.linearize(p, o)
    gc = np.zeros((p.n_cams, 6))
    gp = np.zeros((p.n_points, 3))
    np.add.at(gc, p.obs_cam, 2 * w[:, None] * np.einsum("nrk,nr->nk", jc, e))
    np.add.at(gp, p.obs_point, 2 * w[:, None] * np.einsum("nrk,nr->nk", jp, e))
    free_c = p.cam_fixed == 0
    assert vrel(g["cam_tangent"][free_c], gc[free_c]) < 1e-10
    assert np.all(g["cam_tangent"][~free_c] == 0)
    assert vrel(g["points"], gp) < 1e-10
    assert vrel(g["obs_uv"], 2 * w[:, None] * e) < 1e-10
    # intrinsics: d e / d (fx, fy, cx, cy) = -(x/z, 0), -(0, y/z), -(1, 0), -(0, 1)
    R = p.cam_pose[:, [0, 1, 2, 4, 5, 6, 8, 9, 10]].reshape(-1, 3, 3)
    t = p.cam_pose[:, [3, 7, 11]]
    Xc = np.einsum("nij,nj->ni", R[p.obs_cam], p.points[p.obs_point]) + t[p.obs_cam]
    we = 2 * w[:, None] * e
    gk = -np.array([np.sum(we[:, 0] * Xc[:, 0] / Xc[:, 2]), np.sum(we[:, 1] * Xc[:, 1] / Xc[:, 2]),
                    np.sum(we[:, 0]), np.sum(we[:, 1])])
    assert vrel(g["intrinsics"], gk) < 1e-10


def fd_check(ctx, p, o, n, seed, replay, tol):
    r, lam, _ = ctx.vjp(p, o)
    cb, pb, xb = upstream(p, seed)
    _, _, g = ctx.vjp(p, o, lam, cost_bar=cb, pose_bar=pb, point_bar=xb)
    h = 1e-6
    ks = coords(p, n, seed + 1)
    fd, an = [], []
    for k in ks:
        v = theta_of(p, k)
        lp = loss(replay(with_theta(p, k, v + h), lam), cb, pb, xb)
        lm = loss(replay(with_theta(p, k, v - h), lam), cb, pb, xb)
        fd.append((lp - lm) / (2 * h))
        an.append(grad_of(g, k))
    err = vrel(an, fd)
    assert err < tol, err
    # Coordinate by coordinate.  The step-1e-6 difference carries ~1e-16 |L| / h of rounding noise
    # (~1e-7 here), as large as tol |g_k| for the small coordinates, so each coordinate is checked
    # against the fourth-order central difference (8 (L(+h) - L(-h)) - (L(+2h) - L(-2h))) / 12h with
    # h = 1e-4: |g_k - fd_k| <= tol max(|fd_k|, 1e-2 max |fd|).
    h4 = 1e-4
    fd4 = []
    for k in ks:
        v = theta_of(p, k)
        Ls = [loss(replay(with_theta(p, k, v + s * h4), lam), cb, pb, xb) for s in (1, -1, 2, -2)]
        fd4.append((8.0 * (Ls[0] - Ls[1]) - (Ls[2] - Ls[3])) / (12.0 * h4))
    an, fd4 = np.asarray(an), np.asarray(fd4)
    bad = np.abs(an - fd4) > tol * np.maximum(np.abs(fd4), 1e-2 * np.max(np.abs(fd4)))
    assert not bad.any(), (np.asarray(ks)[bad], an[bad], fd4[bad])
    return err


def test_vjp_matches_central_differences_full_size(ctx):
    """The sphere-cap workload at full size: 200 coordinates, GPU replay."""
    p = Synth(3).window(0)
    o = workload_options(3)

    def replay(q, lam):
        return ctx.vjp(q, o, lam)[0]

    fd_check(ctx, p, o, 200, 5, replay, 1e-5)


def test_vjp_matches_oracle_central_differences(ctx):
    """Finite differences of the oracle's replay (the CPU restatement of the same steps)."""
    p = small()
    o = workload_options(3)

    def replay(q, lam):
        return oracle.solve_schedule(q, o, lam, n_threads=8)[0]

    fd_check(ctx, p, o, 40, 9, replay, 1e-5)


@pytest.mark.parametrize("dtype", ["float64", "float32"])
def test_torch_autograd_function(ctx, dtype):
    torch = pytest.importorskip("torch")
    from nav24_gb300.autograd import bundle_adjust
    p = small()
    o = workload_options(3)
    dt = getattr(torch, dtype)
    uv = torch.tensor(p.obs_uv, dtype=dt, requires_grad=True)
    k4 = torch.tensor(p.intrinsics[:4], dtype=torch.float64, requires_grad=True)
    q = p.copy()
    q.obs_uv = uv.detach().double().numpy()  # the observations the layer sees
    cost, poses, points = bundle_adjust(uv, k4, q, o, ctx)
    cb, pb, xb = upstream(p, 3)
    L = cb * cost + (torch.from_numpy(pb) * poses).sum() + (torch.from_numpy(xb) * points).sum()
    L.backward()
    assert uv.grad.dtype == dt and k4.grad.dtype == torch.float64
    r, lam, _ = ctx.vjp(q, o)
    _, _, g = ctx.vjp(q, o, lam, cost_bar=cb, pose_bar=pb, point_bar=xb)
    tol = 1e-12 if dtype == "float64" else 1e-6
    assert vrel(uv.grad.double().numpy(), g["obs_uv"]) < tol
    assert vrel(k4.grad.numpy(), g["intrinsics"]) < 1e-12
    assert rel(float(cost.detach()), r.stats["final_cost"]) < 1e-14
