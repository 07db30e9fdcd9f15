// vjp_device.cuh - device code of the backward pass through unrolled LM steps (FP64).
//
// One accepted LM step is x' = x [+] dx with dx = (H(x) + lambda I)^-1 b(x), b = -J^T W e,
// H = J^T W J (g2o's first-order robust weighting, W = rho'(e^T e)), [+] the vertex updates
// (T' = exp(dx_c) T as in g2o's VertexSE3Expmap, X' = X + dx_p).  With lambda frozen, the adjoint
// of a step given xbar' is
//   dxbar_c = J_l(dx_c)^T xbar'_c,  dxbar_p = xbar'_p          (through [+])
//   xbar_c  = Ad(exp dx_c)^T xbar'_c + grad psi,  xbar_p = xbar'_p + grad psi
//   u = (H + lambda I)^-1 dxbar                                  (adjoint solve, same factor)
//   psi(x, theta) = -u^T (H(x) dx + g(x)) with u, dx held fixed, g = -b = J^T W e,
// and psi, like the cost, is a sum over edges of terms that need only the edge's residual,
// projection Jacobian and Huber weight: J u = -Jpi v_u with v_u = u_w x Xc + u_v + R u_p, so
// psi_e = -w(s) (Jpi v_u)^T (Jpi v_dx - e).  Every derivative below is of that closed form;
// poses are differentiated through left perturbations T -> exp(eps) T, eps = [alpha; beta].
#pragma once

#include "lm_device.cuh"

namespace navba {
namespace {

constexpr unsigned kVjpFull = 0xffffffffu;

__device__ __forceinline__ void vcross(const double* a, const double* b, double* o) {
    o[0] = a[1] * b[2] - a[2] * b[1];
    o[1] = a[2] * b[0] - a[0] * b[2];
    o[2] = a[0] * b[1] - a[1] * b[0];
}

// ---- dual numbers for the derivative of the SE(3) exponential -----------------------------

struct Dual {
    double v, d;
};
__device__ __forceinline__ Dual operator+(Dual a, Dual b) { return {a.v + b.v, a.d + b.d}; }
__device__ __forceinline__ Dual operator-(Dual a, Dual b) { return {a.v - b.v, a.d - b.d}; }
__device__ __forceinline__ Dual operator*(Dual a, Dual b) { return {a.v * b.v, a.d * b.v + a.v * b.d}; }
__device__ __forceinline__ Dual operator/(Dual a, Dual b) {
    const double q = a.v / b.v;
    return {q, (a.d - q * b.d) / b.v};
}
__device__ __forceinline__ Dual dconst(double v) { return {v, 0.0}; }

// R and V of g2o's SE3Quat::exp on dual numbers, with the branch taken on the value, exactly as
// se3_left_update takes it (small-angle branch R = V = I + W + W^2 below |omega| = 1e-5).
__device__ void exp_rv_dual(const Dual* w, Dual* R, Dual* V) {
    const Dual W[9] = {dconst(0), dconst(0) - w[2], w[1], w[2], dconst(0), dconst(0) - w[0],
                       dconst(0) - w[1], w[0], dconst(0)};
    Dual W2[9];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) W2[i * 3 + j] = W[i * 3] * W[j] + W[i * 3 + 1] * W[3 + j] + W[i * 3 + 2] * W[6 + j];
    const Dual th2 = w[0] * w[0] + w[1] * w[1] + w[2] * w[2];
    const double thv = sqrt(th2.v);
    if (thv < 0.00001) {
        for (int k = 0; k < 9; ++k) R[k] = dconst((k % 4) == 0 ? 1.0 : 0.0) + W[k] + W2[k];
        for (int k = 0; k < 9; ++k) V[k] = R[k];
    } else {
        const Dual th = {thv, th2.d / (2.0 * thv)};
        double s, c;
        sincos(thv, &s, &c);
        const Dual sn = {s, c * th.d}, cs = {c, -s * th.d};
        const Dual a = sn / th;
        const Dual b = (dconst(1.0) - cs) / (th * th);
        const Dual cc = (th - sn) / (th * th * th);
        for (int k = 0; k < 9; ++k) R[k] = dconst((k % 4) == 0 ? 1.0 : 0.0) + a * W[k] + b * W2[k];
        for (int k = 0; k < 9; ++k) V[k] = dconst((k % 4) == 0 ? 1.0 : 0.0) + b * W[k] + cc * W2[k];
    }
}

// Per free camera a: given xbar' (left-tangent adjoint at T' = exp(dx) T), write
//   rc[a]   = J_l(dx)^T xbar'   (adjoint of the step dx through the update), and
//   xcur[a] = Ad(exp dx)^T xbar' (adjoint of T through the update with dx held fixed).
// Column j of J_l is (alpha_j, beta_j): alpha_j = vee(skew(dR_j R^T)), beta_j = d(V ups)_j -
// alpha_j x (V ups), the left-tangent motion of exp(dx) when dx moves along e_j.  The skew part
// is taken because the small-angle R is orthogonal only to O(|omega|^2); the rotation that the
// update applies (R through a normalized quaternion) moves like that skew part.
__global__ void k_vjp_cams_step(const double* dx, const double* xnext, double* rc, double* xcur, int nfc) {
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= nfc) return;
    const double* d = dx + 6 * a;
    const double* xb = xnext + 6 * a;
    double Rv[9], tv[3];
    for (int j = 0; j < 6; ++j) {
        Dual w[3], ups[3], R[9], V[9];
        for (int k = 0; k < 3; ++k) {
            w[k] = {d[k], j == k ? 1.0 : 0.0};
            ups[k] = {d[3 + k], j == 3 + k ? 1.0 : 0.0};
        }
        exp_rv_dual(w, R, V);
        Dual t[3];
        for (int i = 0; i < 3; ++i) t[i] = V[i * 3] * ups[0] + V[i * 3 + 1] * ups[1] + V[i * 3 + 2] * ups[2];
        // M = dR R^T
        double M[9];
        for (int i = 0; i < 3; ++i)
            for (int k = 0; k < 3; ++k)
                M[i * 3 + k] = R[i * 3].d * R[k * 3].v + R[i * 3 + 1].d * R[k * 3 + 1].v + R[i * 3 + 2].d * R[k * 3 + 2].v;
        const double al[3] = {0.5 * (M[7] - M[5]), 0.5 * (M[2] - M[6]), 0.5 * (M[3] - M[1])};
        const double t0[3] = {t[0].v, t[1].v, t[2].v};
        double axt[3];
        vcross(al, t0, axt);
        const double be[3] = {t[0].d - axt[0], t[1].d - axt[1], t[2].d - axt[2]};
        rc[6 * a + j] = xb[0] * al[0] + xb[1] * al[1] + xb[2] * al[2] + xb[3] * be[0] + xb[4] * be[1] + xb[5] * be[2];
        if (j == 0) {
            for (int k = 0; k < 9; ++k) Rv[k] = R[k].v;
            tv[0] = t0[0]; tv[1] = t0[1]; tv[2] = t0[2];
        }
    }
    // the rotation the update applies: R through a normalized quaternion
    double q[4], Re[9];
    q_from_rot(Rv, q);
    q_normalize(q);
    rot_from_q(q, Re);
    // Ad(exp dx) eps = (Re alpha, [t]x Re alpha + Re beta)  =>  Ad^T xbar' = (Re^T (xa + xb x t), Re^T xb)
    double bxt[3];
    vcross(xb + 3, tv, bxt);
    const double s[3] = {xb[0] + bxt[0], xb[1] + bxt[1], xb[2] + bxt[2]};
    for (int k = 0; k < 3; ++k) {
        xcur[6 * a + k] = Re[k] * s[0] + Re[3 + k] * s[1] + Re[6 + k] * s[2];
        xcur[6 * a + 3 + k] = Re[k] * xb[3] + Re[3 + k] * xb[4] + Re[6 + k] * xb[5];
    }
}

// Left-tangent adjoint of each free camera from the cotangent of its output pose entries
// (row-major [R | t]): dR = [alpha]x R, dt = alpha x t + beta  =>  alpha_bar = vee(G R^T - R G^T)
// + t x g_t, beta_bar = g_t.  Zero when pose_bar is null.
__global__ void k_vjp_seed_cams(const CamState* cams, const int32_t* cam_free, int nc, const double* pose_bar,
                                double* cbar) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nc) return;
    const int a = cam_free[k];
    if (a < 0) return;
    double o[6] = {0, 0, 0, 0, 0, 0};
    if (pose_bar) {
        const double* P = pose_bar + 12LL * k;
        const double G[9] = {P[0], P[1], P[2], P[4], P[5], P[6], P[8], P[9], P[10]};
        const double gt[3] = {P[3], P[7], P[11]};
        const double* R = cams[k].R;
        double M[9];  // G R^T
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) M[i * 3 + j] = G[i * 3] * R[j * 3] + G[i * 3 + 1] * R[j * 3 + 1] + G[i * 3 + 2] * R[j * 3 + 2];
        double txg[3];
        vcross(cams[k].t, gt, txg);
        o[0] = M[7] - M[5] + txg[0];
        o[1] = M[2] - M[6] + txg[1];
        o[2] = M[3] - M[1] + txg[2];
        o[3] = gt[0];
        o[4] = gt[1];
        o[5] = gt[2];
    }
    for (int r = 0; r < 6; ++r) cbar[6 * a + r] = o[r];
}

__global__ void k_vjp_seed_points(const double* point_bar, int np, double* pbar) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= np) return;
    for (int j = 0; j < 3; ++j) pbar[4LL * p + j] = point_bar ? point_bar[3LL * p + j] : 0.0;
    pbar[4LL * p + 3] = 0.0;
}

__global__ void k_vjp_axpy(double* y, const double* x, double alpha, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] += alpha * x[i];
}

// ---- per-edge adjoint ---------------------------------------------------------------------

// Adjoint of F = cb * rho(s) + psi_e for one edge (pinhole), with
//   Xc = R X + t, e = z - pi(Xc), s = e^T e, a = Jpi v_u, b = Jpi v_d - e, psi_e = -w(s) a^T b.
// uc/dc: the step vectors of the edge's camera (null: fixed), up/dp: of its point (null: fixed).
struct EdgeAdj {
    double z[2];     // dF / d z
    double k[4];     // dF / d (fx, fy, cx, cy)
    double cam[6];   // dF / d (alpha, beta) of the camera
    double pt[3];    // dF / d X
};

__device__ void edge_adjoint(const Intr& in, const double* R, const double* t, const double* X, const double* z,
                             bool robust, double delta, const double* uc, const double* up, const double* dc,
                             const double* dp, double cb, EdgeAdj& o) {
    double Xc[3];
    transform<double>(R, t, X, Xc);
    const double x = Xc[0], y = Xc[1], zz = Xc[2];
    const double fx = in.fx, fy = in.fy;
    const double iz = 1.0 / zz, iz2 = iz * iz;
    const double xn = x * iz, yn = y * iz;
    const double e0 = z[0] - (fx * xn + in.cx), e1 = z[1] - (fy * yn + in.cy);
    const double s = e0 * e0 + e1 * e1;
    double w = 1.0, wp = 0.0;  // rho'(s), rho''(s)
    if (robust && s > delta * delta) {
        const double r = sqrt(s);
        w = delta / r;
        wp = -0.5 * w / s;
    }
    const double J00 = fx * iz, J02 = -fx * xn * iz, J11 = fy * iz, J12 = -fy * yn * iz;
    double vu[3] = {0, 0, 0}, vd[3] = {0, 0, 0}, Ru[3] = {0, 0, 0}, Rd[3] = {0, 0, 0};
    if (up) {
        for (int i = 0; i < 3; ++i) Ru[i] = R[i * 3] * up[0] + R[i * 3 + 1] * up[1] + R[i * 3 + 2] * up[2];
    }
    if (dp) {
        for (int i = 0; i < 3; ++i) Rd[i] = R[i * 3] * dp[0] + R[i * 3 + 1] * dp[1] + R[i * 3 + 2] * dp[2];
    }
    if (uc) {
        vcross(uc, Xc, vu);
        for (int i = 0; i < 3; ++i) vu[i] += uc[3 + i];
    }
    if (dc) {
        vcross(dc, Xc, vd);
        for (int i = 0; i < 3; ++i) vd[i] += dc[3 + i];
    }
    for (int i = 0; i < 3; ++i) {
        vu[i] += Ru[i];
        vd[i] += Rd[i];
    }
    const double a0 = J00 * vu[0] + J02 * vu[2], a1 = J11 * vu[1] + J12 * vu[2];
    const double b0 = J00 * vd[0] + J02 * vd[2] - e0, b1 = J11 * vd[1] + J12 * vd[2] - e1;
    // reverse sweep
    const double sbar = cb * w - (a0 * b0 + a1 * b1) * wp;
    const double ab0 = -w * b0, ab1 = -w * b1;  // abar
    const double bb0 = -w * a0, bb1 = -w * a1;  // bbar
    const double eb0 = 2.0 * sbar * e0 - bb0, eb1 = 2.0 * sbar * e1 - bb1;
    o.z[0] = eb0;
    o.z[1] = eb1;
    const double pb0 = -eb0, pb1 = -eb1;  // pibar
    // Jpi_bar = abar v_u^T + bbar v_d^T (entries 00, 02, 11, 12)
    const double M00 = ab0 * vu[0] + bb0 * vd[0], M02 = ab0 * vu[2] + bb0 * vd[2];
    const double M11 = ab1 * vu[1] + bb1 * vd[1], M12 = ab1 * vu[2] + bb1 * vd[2];
    // intrinsics: through pi and through Jpi
    o.k[0] = pb0 * xn + M00 * iz - M02 * xn * iz;
    o.k[1] = pb1 * yn + M11 * iz - M12 * yn * iz;
    o.k[2] = pb0;
    o.k[3] = pb1;
    // Xc_bar: through pi (Jpi^T pibar), through Jpi, and through v_u, v_d (u_w x Xc)
    double Xb[3];
    Xb[0] = J00 * pb0 - fx * iz2 * M02;
    Xb[1] = J11 * pb1 - fy * iz2 * M12;
    Xb[2] = J02 * pb0 + J12 * pb1 - fx * iz2 * M00 + 2.0 * fx * xn * iz2 * M02 - fy * iz2 * M11 +
            2.0 * fy * yn * iz2 * M12;
    const double vbu[3] = {J00 * ab0, J11 * ab1, J02 * ab0 + J12 * ab1};  // Jpi^T abar
    const double vbd[3] = {J00 * bb0, J11 * bb1, J02 * bb0 + J12 * bb1};  // Jpi^T bbar
    double tmp[3];
    if (uc) {
        vcross(vbu, uc, tmp);
        for (int i = 0; i < 3; ++i) Xb[i] += tmp[i];
    }
    if (dc) {
        vcross(vbd, dc, tmp);
        for (int i = 0; i < 3; ++i) Xb[i] += tmp[i];
    }
    // pose: Xc' = Xc + alpha x Xc + beta, R' u = R u + alpha x (R u)
    double al[3];
    vcross(Xc, Xb, al);
    vcross(Ru, vbu, tmp);
    for (int i = 0; i < 3; ++i) al[i] += tmp[i];
    vcross(Rd, vbd, tmp);
    for (int i = 0; i < 3; ++i) al[i] += tmp[i];
    o.cam[0] = al[0]; o.cam[1] = al[1]; o.cam[2] = al[2];
    o.cam[3] = Xb[0]; o.cam[4] = Xb[1]; o.cam[5] = Xb[2];
    // point: Xc = R X + t
    for (int k = 0; k < 3; ++k) o.pt[k] = R[k] * Xb[0] + R[3 + k] * Xb[1] + R[6 + k] * Xb[2];
}

// Block sums of 4 per-thread values; thread 0 writes out[4 * blockIdx.x + k].
__device__ void vjp_block_sum4(double (&v)[4], double* out) {
    __shared__ double red[32 * 4];
#pragma unroll
    for (int k = 0; k < 4; ++k)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_down_sync(kVjpFull, v[k], o);
    if ((threadIdx.x & 31) == 0)
#pragma unroll
        for (int k = 0; k < 4; ++k) red[4 * (threadIdx.x >> 5) + k] = v[k];
    __syncthreads();
    if (threadIdx.x == 0)
        for (int k = 0; k < 4; ++k) {
            double r = 0.0;
            for (int i = 0; i < (int)(blockDim.x >> 5); ++i) r += red[4 * i + k];
            out[4 * blockIdx.x + k] = r;
        }
}

// Thread per point over its edges (point-major): adds each edge's dF/dz to uvbar, its dF/dX to the
// point's adjoint pbar (free points), writes its camera adjoint to ecam[8 e] (free cameras) and
// block sums of dF/d(fx, fy, cx, cy) to part[4 block].  camr: FP64 [R|t] (12 per camera) of the
// state; uc/dc: 6 per free camera; up/dp: 4 per point (null: the step terms are absent).
__global__ void k_vjp_edges(WinArgs<double> A, int np, const double* camr, const double* X, const double* uc,
                            const double* up, const double* dc, const double* dp, double cb, double* pbar, double* ecam,
                            double* uvbar, double* part) {
    double kacc[4] = {0, 0, 0, 0};
    const int CT = gridDim.x * blockDim.x;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < np; p += CT) {
        const bool fp = A.pt_free[p] >= 0;
        const double Xp[3] = {X[4LL * p], X[4LL * p + 1], X[4LL * p + 2]};
        double ps[3] = {0, 0, 0};
        for (int e = A.pt_eoff[p]; e < A.pt_eoff[p + 1]; ++e) {
            const int a = A.edge_fc[e];
            const double* cr = camr + 12LL * A.edge_cam[e];
            const double z[2] = {A.edge_uv[2LL * e], A.edge_uv[2LL * e + 1]};
            EdgeAdj o;
            edge_adjoint(A.intr, cr, cr + 9, Xp, z, A.lm.robust != 0, A.lm.huber_delta,
                         (uc && a >= 0) ? uc + 6LL * a : nullptr, (up && fp) ? up + 4LL * p : nullptr,
                         (dc && a >= 0) ? dc + 6LL * a : nullptr, (dp && fp) ? dp + 4LL * p : nullptr, cb, o);
            uvbar[2LL * e] += o.z[0];
            uvbar[2LL * e + 1] += o.z[1];
            for (int k = 0; k < 4; ++k) kacc[k] += o.k[k];
            for (int k = 0; k < 3; ++k) ps[k] += o.pt[k];
            if (a >= 0)
                for (int k = 0; k < 6; ++k) ecam[8LL * e + k] = o.cam[k];
        }
        if (fp)
            for (int k = 0; k < 3; ++k) pbar[4LL * p + k] += ps[k];
    }
    vjp_block_sum4(kacc, part);
}

// Warp per work item (free camera, chunk of its camera-major edge list): sum of the chunk's edge
// vectors src[8 e .. 8 e + 5] -> ipart[8 item].  With `lt` set, the edge vector is A_e t_p instead
// (A_e = W_e L_p^T of the factorization, t_p = src[4 p .. 4 p + 2]); edges of fixed points add 0.
__global__ void k_vjp_cam_items(WinArgs<double> A, const int4* items, int n_items, const int32_t* cam_list,
                                const double* src, bool lt, double* ipart) {
    const int lane = threadIdx.x & 31;
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int CW = (gridDim.x * blockDim.x) >> 5;
    for (int it = gw; it < n_items; it += CW) {
        const int4 wi = items[it];
        double s[6] = {0, 0, 0, 0, 0, 0};
        for (int i = lane; i < wi.z; i += 32) {
            const int e = cam_list[wi.y + i];
            if (lt) {
                const int p = A.edge_pt[e];
                if (A.pt_free[p] < 0) continue;
                double Ae[18];
                Rec<double>::load18(A.edge_a + 18LL * e, Ae);
                const double t0 = src[4LL * p], t1 = src[4LL * p + 1], t2 = src[4LL * p + 2];
                for (int r = 0; r < 6; ++r) s[r] += Ae[r * 3] * t0 + Ae[r * 3 + 1] * t1 + Ae[r * 3 + 2] * t2;
            } else {
                for (int r = 0; r < 6; ++r) s[r] += src[8LL * e + r];
            }
        }
#pragma unroll
        for (int r = 0; r < 6; ++r)
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) s[r] += __shfl_xor_sync(kVjpFull, s[r], o);
        if (lane < 6) {
#pragma unroll
            for (int r = 0; r < 6; ++r)
                if (r == lane) ipart[8LL * it + r] = s[r];
        }
    }
}

// Per free point: tr_p = L_p r_p (L lower triangular, (V_p + lambda I)^-1 = L^T L); 0 for fixed.
__global__ void k_vjp_lt_points(WinArgs<double> A, int np, const double* rp, double* tr) {
    const int CT = gridDim.x * blockDim.x;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < np; p += CT) {
        double o[3] = {0, 0, 0};
        if (A.pt_free[p] >= 0) {
            double lt[12];
            Rec<double>::load12(A.pt_lt + 12LL * p, lt);
            const double r0 = rp[4LL * p], r1 = rp[4LL * p + 1], r2 = rp[4LL * p + 2];
            o[0] = lt[0] * r0;
            o[1] = lt[1] * r0 + lt[2] * r1;
            o[2] = lt[3] * r0 + lt[4] * r1 + lt[5] * r2;
        }
        tr[4LL * p] = o[0];
        tr[4LL * p + 1] = o[1];
        tr[4LL * p + 2] = o[2];
        tr[4LL * p + 3] = 0.0;
    }
}

// Per free point: y_p = L_p^T (t_p - sum_e A_e^T y_c(e)) over its edges with a free camera; t_p is
// tsrc[tstride p + toff ..]; 0 for fixed points.  (The back-substitution of the Schur solve.)
__global__ void k_vjp_point_solve(WinArgs<double> A, int np, const double* tsrc, int tstride, int toff,
                                  const double* yc, double* yp) {
    const int CT = gridDim.x * blockDim.x;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < np; p += CT) {
        double d[3] = {0, 0, 0};
        if (A.pt_free[p] >= 0) {
            double lt[12];
            Rec<double>::load12(A.pt_lt + 12LL * p, lt);
            const double* t = tsrc + (long long)tstride * p + toff;
            double u0 = t[0], u1 = t[1], u2 = t[2];
            for (int e = A.pt_eoff[p]; e < A.pt_eoff[p + 1]; ++e) {
                const int a = A.edge_fc[e];
                if (a < 0) continue;
                double Ae[18];
                Rec<double>::load18(A.edge_a + 18LL * e, Ae);
                for (int r = 0; r < 6; ++r) {
                    const double y = yc[6 * a + r];
                    u0 -= Ae[r * 3] * y;
                    u1 -= Ae[r * 3 + 1] * y;
                    u2 -= Ae[r * 3 + 2] * y;
                }
            }
            d[0] = lt[0] * u0 + lt[1] * u1 + lt[3] * u2;
            d[1] = lt[2] * u1 + lt[4] * u2;
            d[2] = lt[5] * u2;
        }
        yp[4LL * p] = d[0];
        yp[4LL * p + 1] = d[1];
        yp[4LL * p + 2] = d[2];
        yp[4LL * p + 3] = 0.0;
    }
}

}  // namespace
}  // namespace navba
