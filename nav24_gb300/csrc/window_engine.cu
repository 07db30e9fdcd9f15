// window_engine.cu - batched bundle adjustment: one persistent kernel solves many windows.
//
// Each CTA takes windows from a work queue (the host orders it, largest first) and runs the
// whole Levenberg-Marquardt loop of one window before taking the next, so a batch of uneven
// windows is a single launch.  Per window the CTA keeps the camera states, the camera blocks
// of H and the reduced camera system S in shared memory; per-point and per-edge quantities
// stream through global memory (L2-resident for a window).
//
// One LM iteration (g2o OptimizationAlgorithmLevenberg::solve semantics, as used by nav24's
// GraphOptim::solve, core/backEnd/BE_GraphOptim.cpp:67-68):
//   linearize  thread per point: e, J_pose, J_point, Huber weight per edge
//              (EdgeSE3ProjectXYZ::computeError/linearizeOplus, OptimizableTypes.hpp:102-107,
//              OptimizableTypes.cpp:140-161); V_p, g_p in registers; W_e = w Jc^T Jp stored;
//              warp per camera over its edge list: U_c, g_c by warp-shuffle reduction.
//   trial      Vinv_p = (V_p + lambda I)^-1, Y_e = W_e Vinv_p (thread per point);
//              S_ab = [a==b](U_a + lambda I) - sum Y_i W_j^T, one warp per 6x6 block, summed
//              in registers and reduced by shuffles (no atomics, fixed order);
//              FP64 Cholesky of S in shared memory; dx_p by back-substitution; T <- exp(dx) T;
//              cost of the trial state; gain ratio, accept/reject, damping update.
// Real is double (plain FP64 form) or float (mixed form: residuals, Jacobians and Hessian
// blocks in FP32; S, its Cholesky, the states, the SE(3) update and the cost sums in FP64).
#include <algorithm>
#include <cfloat>

#include "engine.hpp"

namespace navba {
namespace {

constexpr unsigned kFull = 0xffffffffu;

struct SmemHead {
    CamState cams[2][kWinMaxCams];
    double U[kWinMaxFreeCams][28];  // packed lower U (21) | g_c (6) | pad
    double red[66];
    int32_t fcam[kWinMaxFreeCams];
    int32_t loff[kWinMaxCams + 1];
    int32_t lcnt[kWinMaxCams];
    double lambda, nu, chi, chi_new, scale, maxdiag;
    int32_t cur, ok, win, pad;
};

template <class Real>
struct WinArgs {
    const WinDesc* win;
    int32_t n_win;
    const int32_t* order;
    int32_t* queue;
    const CamState* cam_init;
    const int32_t* cam_free;
    const double* pt_init;
    const int32_t* pt_free;
    const int32_t* pt_eoff;
    const int32_t* edge_cam;
    const int32_t* edge_pt;
    const double* edge_uv;
    double* x[2];
    Real* pt_vg;
    Real* pt_vinv;
    Real* edge_jce;
    Real* edge_w;
    Real* edge_y;
    int32_t* cam_list;
    CamState* cam_out;
    double* pt_out;
    double* trace;
    int32_t trace_stride;
    WinStats* stats;
    double* debug;
    double debug_lambda;
    Intr intr;
    LmOptions lm;
    int32_t ld;     // leading dimension of S in shared memory
    int32_t max_m;
};

NAVBA_HD int tri(int r, int c) { return r * (r + 1) / 2 + c; }  // packed lower index, c <= r

__device__ __forceinline__ double block_sum(double v, double* red) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(kFull, v, o);
    __syncthreads();
    if (lane == 0) red[wid] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double r = 0.0;
        for (int i = 0; i < nw; ++i) r += red[i];
        red[64] = r;
    }
    __syncthreads();
    return red[64];
}

__device__ __forceinline__ double block_max(double v, double* red) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(kFull, v, o));
    __syncthreads();
    if (lane == 0) red[wid] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double r = 0.0;
        for (int i = 0; i < nw; ++i) r = fmax(r, red[i]);
        red[64] = r;
    }
    __syncthreads();
    return red[64];
}

template <class Real>
__device__ __forceinline__ void cam_real(const CamState& c, Real* o) {
#pragma unroll
    for (int k = 0; k < 9; ++k) o[k] = (Real)c.R[k];
    o[9] = (Real)c.t[0];
    o[10] = (Real)c.t[1];
    o[11] = (Real)c.t[2];
}

// Robust chi2 of the window for the cameras `camc` (12 values each, precision Cost) and the
// point buffer X.
template <class Cost, class Real>
__device__ double window_cost(const WinArgs<Real>& A, const WinDesc& D, SmemHead& s, const Cost* camc,
                              const double* X) {
    double acc = 0.0;
    const Cost delta = (Cost)A.lm.huber_delta;
    for (int p = threadIdx.x; p < D.npt; p += blockDim.x) {
        const int gp = D.pt0 + p;
        const Cost Xr[3] = {(Cost)X[4LL * gp], (Cost)X[4LL * gp + 1], (Cost)X[4LL * gp + 2]};
        const int e1 = A.pt_eoff[gp + 1];
        for (int e = A.pt_eoff[gp]; e < e1; ++e) {
            const Cost* cr = camc + 12 * A.edge_cam[e];
            const Cost z[2] = {(Cost)A.edge_uv[2LL * e], (Cost)A.edge_uv[2LL * e + 1]};
            acc += edge_cost<Cost>(A.intr, cr, cr + 9, Xr, z, A.lm.robust != 0, delta);
        }
    }
    return block_sum(acc, s.red);
}

// FP64 camera array (12 values per camera) of camera buffer cb, built in `out` (shared).
template <class Real>
__device__ void cams_fp64(const WinDesc& D, const SmemHead& s, int cb, double* out) {
    for (int c = threadIdx.x; c < D.ncam; c += blockDim.x) cam_real<double>(s.cams[cb][c], out + 12 * c);
    __syncthreads();
}

// Camera-major list of the edges of each free camera (stable: point-major order kept).
template <class Real>
__device__ void build_cam_lists(const WinArgs<Real>& A, const WinDesc& D, SmemHead& s) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int c = wid; c < D.ncam; c += nw) {
        int cnt = 0;
        if (A.cam_free[D.cam0 + c] >= 0) {
            for (int base = 0; base < D.ne; base += 32) {
                const int e = base + lane;
                const bool hit = e < D.ne && A.edge_cam[D.e0 + e] == c;
                cnt += __popc(__ballot_sync(kFull, hit));
            }
        }
        if (lane == 0) s.lcnt[c] = cnt;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        int acc = 0;
        for (int c = 0; c < D.ncam; ++c) {
            s.loff[c] = acc;
            acc += s.lcnt[c];
        }
        s.loff[D.ncam] = acc;
        for (int c = 0; c < D.ncam; ++c) {
            const int a = A.cam_free[D.cam0 + c];
            if (a >= 0) s.fcam[a] = c;
        }
    }
    __syncthreads();
    for (int c = wid; c < D.ncam; c += nw) {
        if (A.cam_free[D.cam0 + c] < 0) continue;
        int pos = s.loff[c];
        for (int base = 0; base < D.ne; base += 32) {
            const int e = base + lane;
            const bool hit = e < D.ne && A.edge_cam[D.e0 + e] == c;
            const unsigned m = __ballot_sync(kFull, hit);
            if (hit) A.cam_list[D.e0 + pos + __popc(m & ((1u << lane) - 1u))] = D.e0 + e;
            pos += __popc(m);
        }
    }
    __syncthreads();
}

// Linearize all edges at the current state; fills U, g_c (shared), V_p, g_p, W_e (global).
template <class Real>
__device__ void window_linearize(const WinArgs<Real>& A, const WinDesc& D, SmemHead& s, const Real* camr) {
    const Real delta = (Real)A.lm.huber_delta;
    const double* X = A.x[s.cur];
    double mx = 0.0;
    for (int p = threadIdx.x; p < D.npt; p += blockDim.x) {
        const int gp = D.pt0 + p;
        const bool fp = A.pt_free[gp] >= 0;
        const Real Xr[3] = {(Real)X[4LL * gp], (Real)X[4LL * gp + 1], (Real)X[4LL * gp + 2]};
        Real V[6] = {0, 0, 0, 0, 0, 0}, g[3] = {0, 0, 0};
        const int e1 = A.pt_eoff[gp + 1];
        for (int e = A.pt_eoff[gp]; e < e1; ++e) {
            const int c = A.edge_cam[e];
            const Real* cr = camr + 12 * c;
            const Real z[2] = {(Real)A.edge_uv[2LL * e], (Real)A.edge_uv[2LL * e + 1]};
            EdgeLin<Real> L;
            edge_linearize<Real>(A.intr, cr, cr + 9, Xr, z, A.lm.robust != 0, delta, L);
            Real* jce = A.edge_jce + 16LL * e;
#pragma unroll
            for (int k = 0; k < 12; ++k) jce[k] = L.jc[k];
            jce[12] = L.e[0];
            jce[13] = L.e[1];
            jce[14] = L.w;
            if (fp) {
                const Real w = L.w;
                const Real* jp = L.jp;
                V[0] += w * (jp[0] * jp[0] + jp[3] * jp[3]);
                V[1] += w * (jp[0] * jp[1] + jp[3] * jp[4]);
                V[2] += w * (jp[0] * jp[2] + jp[3] * jp[5]);
                V[3] += w * (jp[1] * jp[1] + jp[4] * jp[4]);
                V[4] += w * (jp[1] * jp[2] + jp[4] * jp[5]);
                V[5] += w * (jp[2] * jp[2] + jp[5] * jp[5]);
                const Real we0 = -w * L.e[0], we1 = -w * L.e[1];
                g[0] += jp[0] * we0 + jp[3] * we1;
                g[1] += jp[1] * we0 + jp[4] * we1;
                g[2] += jp[2] * we0 + jp[5] * we1;
                if (A.cam_free[D.cam0 + c] >= 0) {
                    Real* W = A.edge_w + 18LL * e;
#pragma unroll
                    for (int r = 0; r < 6; ++r)
#pragma unroll
                        for (int k = 0; k < 3; ++k) W[r * 3 + k] = w * (L.jc[r] * jp[k] + L.jc[6 + r] * jp[3 + k]);
                }
            }
        }
        if (fp) {
            Real* vg = A.pt_vg + 12LL * gp;
#pragma unroll
            for (int k = 0; k < 6; ++k) vg[k] = V[k];
            vg[6] = g[0]; vg[7] = g[1]; vg[8] = g[2];
            mx = fmax(mx, fmax(fabs((double)V[0]), fmax(fabs((double)V[3]), fabs((double)V[5]))));
        }
    }
    __syncthreads();
    // camera blocks: warp per free camera, shuffle reduction
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int a = wid; a < D.nfc; a += nw) {
        const int c = s.fcam[a];
        const int* list = A.cam_list + D.e0 + s.loff[c];
        const int cnt = s.lcnt[c];
        Real u[27];
#pragma unroll
        for (int k = 0; k < 27; ++k) u[k] = Real(0);
        for (int i = lane; i < cnt; i += 32) {
            const Real* jce = A.edge_jce + 16LL * list[i];
            Real jc[12];
#pragma unroll
            for (int k = 0; k < 12; ++k) jc[k] = jce[k];
            const Real e0 = jce[12], e1 = jce[13], w = jce[14];
#pragma unroll
            for (int r = 0; r < 6; ++r)
#pragma unroll
                for (int q = 0; q <= r; ++q) u[tri(r, q)] += w * (jc[r] * jc[q] + jc[6 + r] * jc[6 + q]);
            const Real we0 = -w * e0, we1 = -w * e1;
#pragma unroll
            for (int r = 0; r < 6; ++r) u[21 + r] += jc[r] * we0 + jc[6 + r] * we1;
        }
#pragma unroll
        for (int k = 0; k < 27; ++k)
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) u[k] += __shfl_xor_sync(kFull, u[k], o);
#pragma unroll
        for (int k = 0; k < 27; ++k)
            if ((k & 31) == lane) s.U[a][k] = (double)u[k];
        if (lane == 0) {
            double m = 0.0;
#pragma unroll
            for (int r = 0; r < 6; ++r) m = fmax(m, fabs((double)u[tri(r, r)]));
            mx = fmax(mx, m);
        }
    }
    const double m = block_max(mx, s.red);
    if (threadIdx.x == 0) s.maxdiag = m;
    __syncthreads();
}

// Reduced camera system for damping lambda: S (lower blocks, shared) and b' (shared).
template <class Real>
__device__ void window_schur(const WinArgs<Real>& A, const WinDesc& D, SmemHead& s, double lambda,
                             double* S, double* bs) {
    const Real lam = (Real)lambda;
    for (int p = threadIdx.x; p < D.npt; p += blockDim.x) {
        const int gp = D.pt0 + p;
        if (A.pt_free[gp] < 0) continue;
        const Real* vg = A.pt_vg + 12LL * gp;
        Real V[6] = {vg[0] + lam, vg[1], vg[2], vg[3] + lam, vg[4], vg[5] + lam};
        Real Vi[6];
        inv_sym3<Real>(V, Vi);
        Real* vi = A.pt_vinv + 8LL * gp;
#pragma unroll
        for (int k = 0; k < 6; ++k) vi[k] = Vi[k];
        const Real M[9] = {Vi[0], Vi[1], Vi[2], Vi[1], Vi[3], Vi[4], Vi[2], Vi[4], Vi[5]};
        const int e1 = A.pt_eoff[gp + 1];
        for (int e = A.pt_eoff[gp]; e < e1; ++e) {
            if (A.cam_free[D.cam0 + A.edge_cam[e]] < 0) continue;
            const Real* W = A.edge_w + 18LL * e;
            Real* Y = A.edge_y + 18LL * e;
#pragma unroll
            for (int r = 0; r < 6; ++r) {
                const Real w0 = W[r * 3 + 0], w1 = W[r * 3 + 1], w2 = W[r * 3 + 2];
#pragma unroll
                for (int k = 0; k < 3; ++k) Y[r * 3 + k] = w0 * M[k] + w1 * M[3 + k] + w2 * M[6 + k];
            }
        }
    }
    __syncthreads();
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int nblk = D.nfc * (D.nfc + 1) / 2;
    const int ld = A.ld;
    for (int blk = wid; blk < nblk; blk += nw) {
        int a = (int)((sqrt(8.0 * blk + 1.0) - 1.0) * 0.5);
        while ((a + 1) * (a + 2) / 2 <= blk) ++a;
        while (a * (a + 1) / 2 > blk) --a;
        const int b = blk - a * (a + 1) / 2;
        const int ca = s.fcam[a], cb = s.fcam[b];
        const int* list = A.cam_list + D.e0 + s.loff[ca];
        const int cnt = s.lcnt[ca];
        Real acc[36];
        Real accb[6];
#pragma unroll
        for (int k = 0; k < 36; ++k) acc[k] = Real(0);
#pragma unroll
        for (int k = 0; k < 6; ++k) accb[k] = Real(0);
        for (int i = lane; i < cnt; i += 32) {
            const int ei = list[i];
            const int gp = D.pt0 + A.edge_pt[ei];
            if (A.pt_free[gp] < 0) continue;
            const Real* Y = A.edge_y + 18LL * ei;
            Real y[18];
#pragma unroll
            for (int k = 0; k < 18; ++k) y[k] = Y[k];
            if (a == b) {
                const Real* g = A.pt_vg + 12LL * gp + 6;
                const Real g0 = g[0], g1 = g[1], g2 = g[2];
#pragma unroll
                for (int r = 0; r < 6; ++r) accb[r] += y[r * 3 + 0] * g0 + y[r * 3 + 1] * g1 + y[r * 3 + 2] * g2;
            }
            const int e1 = A.pt_eoff[gp + 1];
            for (int ej = A.pt_eoff[gp]; ej < e1; ++ej) {
                if (A.edge_cam[ej] != cb) continue;
                const Real* W = A.edge_w + 18LL * ej;
                Real wv[18];
#pragma unroll
                for (int k = 0; k < 18; ++k) wv[k] = W[k];
#pragma unroll
                for (int r = 0; r < 6; ++r)
#pragma unroll
                    for (int q = 0; q < 6; ++q)
                        acc[r * 6 + q] += y[r * 3 + 0] * wv[q * 3 + 0] + y[r * 3 + 1] * wv[q * 3 + 1] + y[r * 3 + 2] * wv[q * 3 + 2];
            }
        }
#pragma unroll
        for (int k = 0; k < 36; ++k)
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) acc[k] += __shfl_xor_sync(kFull, acc[k], o);
        if (a == b) {
#pragma unroll
            for (int k = 0; k < 6; ++k)
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) accb[k] += __shfl_xor_sync(kFull, accb[k], o);
        }
#pragma unroll
        for (int k = 0; k < 36; ++k) {
            if ((k & 31) != lane) continue;
            const int r = k / 6, q = k % 6;
            double v = -(double)acc[k];
            if (a == b) {
                v += s.U[a][r >= q ? tri(r, q) : tri(q, r)];
                if (r == q) v += lambda;
            }
            S[(6 * a + r) * ld + 6 * b + q] = v;
        }
        if (a == b && lane < 6) {
#pragma unroll
            for (int k = 0; k < 6; ++k)
                if (k == lane) bs[6 * a + k] = s.U[a][21 + k] - (double)accb[k];
        }
    }
    __syncthreads();
}

// In-place Cholesky (LL^T) of the lower triangle of S (m x m, leading dimension ld), FP64.
// Returns false (to all threads) when a pivot is not positive and finite.
__device__ bool smem_cholesky(double* S, int m, int ld, SmemHead& s) {
    if (threadIdx.x == 0) s.ok = 1;
    __syncthreads();
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int j = 0; j < m; ++j) {
        if (threadIdx.x == 0) {
            const double d = S[j * ld + j];
            if (!(d > 0.0) || !isfinite(d)) {
                s.ok = 0;
                S[j * ld + j] = 1.0;
            } else {
                S[j * ld + j] = sqrt(d);
            }
        }
        __syncthreads();
        const double piv = S[j * ld + j];
        for (int i = j + 1 + threadIdx.x; i < m; i += blockDim.x) S[i * ld + j] = S[i * ld + j] / piv;
        __syncthreads();
        for (int i = j + 1 + wid; i < m; i += nw) {
            const double lij = S[i * ld + j];
            for (int k = j + 1 + lane; k <= i; k += 32) S[i * ld + k] -= lij * S[k * ld + j];
        }
        __syncthreads();
    }
    return s.ok != 0;
}

// Solve L L^T x = b in place (warp 0), FP64.
__device__ void smem_chol_solve(const double* L, int m, int ld, double* x) {
    if (threadIdx.x < 32) {
        const int lane = threadIdx.x;
        for (int i = 0; i < m; ++i) {
            double sum = 0.0;
            for (int k = lane; k < i; k += 32) sum += L[i * ld + k] * x[k];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(kFull, sum, o);
            if (lane == 0) x[i] = (x[i] - sum) / L[i * ld + i];
            __syncwarp();
        }
        for (int i = m - 1; i >= 0; --i) {
            double sum = 0.0;
            for (int k = i + 1 + lane; k < m; k += 32) sum += L[k * ld + i] * x[k];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(kFull, sum, o);
            if (lane == 0) x[i] = (x[i] - sum) / L[i * ld + i];
            __syncwarp();
        }
    }
    __syncthreads();
}

// Apply the step: trial cameras (shared) and trial points (global); returns dx^T(lambda dx + b).
template <class Real>
__device__ double window_update(const WinArgs<Real>& A, const WinDesc& D, SmemHead& s, double lambda,
                                const double* dc, Real* camr_trial) {
    const int cur = s.cur, tr = cur ^ 1;
    double sc = 0.0;
    for (int c = threadIdx.x; c < D.ncam; c += blockDim.x) {
        const int a = A.cam_free[D.cam0 + c];
        if (a >= 0) {
            se3_left_update(dc + 6 * a, s.cams[cur][c], s.cams[tr][c]);
#pragma unroll
            for (int r = 0; r < 6; ++r) sc += dc[6 * a + r] * (lambda * dc[6 * a + r] + s.U[a][21 + r]);
        }
        cam_real<Real>(s.cams[tr][c], camr_trial + 12 * c);
    }
    const double* Xc = A.x[cur];
    double* Xt = A.x[tr];
    for (int p = threadIdx.x; p < D.npt; p += blockDim.x) {
        const int gp = D.pt0 + p;
        if (A.pt_free[gp] < 0) continue;
        const Real* vg = A.pt_vg + 12LL * gp;
        Real c3[3] = {vg[6], vg[7], vg[8]};
        const int e1 = A.pt_eoff[gp + 1];
        for (int e = A.pt_eoff[gp]; e < e1; ++e) {
            const int a = A.cam_free[D.cam0 + A.edge_cam[e]];
            if (a < 0) continue;
            const Real* W = A.edge_w + 18LL * e;
#pragma unroll
            for (int r = 0; r < 6; ++r) {
                const Real d = (Real)dc[6 * a + r];
                c3[0] -= W[r * 3 + 0] * d;
                c3[1] -= W[r * 3 + 1] * d;
                c3[2] -= W[r * 3 + 2] * d;
            }
        }
        const Real* vi = A.pt_vinv + 8LL * gp;
        const Real d0 = vi[0] * c3[0] + vi[1] * c3[1] + vi[2] * c3[2];
        const Real d1 = vi[1] * c3[0] + vi[3] * c3[1] + vi[4] * c3[2];
        const Real d2 = vi[2] * c3[0] + vi[4] * c3[1] + vi[5] * c3[2];
        Xt[4LL * gp + 0] = Xc[4LL * gp + 0] + (double)d0;
        Xt[4LL * gp + 1] = Xc[4LL * gp + 1] + (double)d1;
        Xt[4LL * gp + 2] = Xc[4LL * gp + 2] + (double)d2;
        sc += (double)d0 * (lambda * (double)d0 + (double)vg[6]) + (double)d1 * (lambda * (double)d1 + (double)vg[7]) +
              (double)d2 * (lambda * (double)d2 + (double)vg[8]);
    }
    return block_sum(sc, s.red);
}

template <class Real>
__device__ void solve_window(const WinArgs<Real>& A, int w, SmemHead& s, double* S, double* bs, Real* camr,
                             double* camd) {
    const WinDesc D = A.win[w];
    const int m = 6 * D.nfc;
    const int ld = A.ld;
    WinStats* st = A.stats + w;
    double* trace = A.trace + (long long)w * A.trace_stride;
    // initial state: both camera and point buffers hold the initial values
    for (int c = threadIdx.x; c < D.ncam; c += blockDim.x) {
        s.cams[0][c] = A.cam_init[D.cam0 + c];
        s.cams[1][c] = A.cam_init[D.cam0 + c];
        cam_real<Real>(s.cams[0][c], camr + 12 * c);
    }
    for (int p = threadIdx.x; p < D.npt; p += blockDim.x) {
        const long long gp = D.pt0 + p;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            A.x[0][4 * gp + k] = A.pt_init[4 * gp + k];
            A.x[1][4 * gp + k] = A.pt_init[4 * gp + k];
        }
    }
    if (threadIdx.x == 0) s.cur = 0;
    __syncthreads();
    build_cam_lists(A, D, s);
    const bool mixed = sizeof(Real) == 4;
    double chi = window_cost<Real, Real>(A, D, s, camr, A.x[0]);
    double chi0_fp64 = chi;
    if (mixed) {
        cams_fp64<Real>(D, s, 0, camd);
        chi0_fp64 = window_cost<double, Real>(A, D, s, camd, A.x[0]);
    }
    int iters_done = 0, acc = 0, rej = 0, term = NAV_BA_TERM_ITERATIONS;
    double lambda = 0.0, nu = 2.0;
    if (threadIdx.x == 0) trace[0] = chi;
    bool bad = !isfinite(chi);
    if (!bad && D.nfc + D.nfp == 0) term = NAV_BA_TERM_NOTHING_TO_DO;
    if (!bad && term == NAV_BA_TERM_ITERATIONS) {
        Real* camr_tr = camr + 12 * kWinMaxCams;
        for (int it = 0; it < A.lm.iterations; ++it) {
            window_linearize(A, D, s, camr);
            if (it == 0) {
                lambda = A.lm.initial_lambda > 0 ? A.lm.initial_lambda : A.lm.tau * s.maxdiag;
                nu = 2.0;
            }
            double rho = 0.0;
            int q = 0;
            do {
                const double lam_use = (A.debug && it == 0 && q == 0) ? A.debug_lambda : lambda;
                for (int k = threadIdx.x; k < m * ld; k += blockDim.x) S[k] = 0.0;
                __syncthreads();
                window_schur(A, D, s, lam_use, S, bs);
                if (A.debug) {
                    // reduced-system output of window 0: full symmetric S then b'
                    for (int k = threadIdx.x; k < m * m; k += blockDim.x) {
                        const int r = k / m, c = k % m;
                        A.debug[k] = r >= c ? S[r * ld + c] : S[c * ld + r];
                    }
                    for (int k = threadIdx.x; k < m; k += blockDim.x) A.debug[m * m + k] = bs[k];
                    __syncthreads();
                    return;
                }
                const bool ok = smem_cholesky(S, m, ld, s);
                if (ok) {
                    smem_chol_solve(S, m, ld, bs);
                } else {
                    for (int k = threadIdx.x; k < m; k += blockDim.x) bs[k] = 0.0;
                    __syncthreads();
                }
                double scale = window_update(A, D, s, lambda, bs, camr_tr);
                double chi_new = window_cost<Real, Real>(A, D, s, camr_tr, A.x[s.cur ^ 1]);
                if (!ok) chi_new = DBL_MAX;
                rho = chi - chi_new;
                scale += 1e-3;
                rho /= scale;
                const bool accept = rho > 0 && isfinite(chi_new);
                if (accept) {
                    double alpha = 1.0 - pow(2 * rho - 1, 3.0);
                    alpha = fmin(alpha, 2.0 / 3.0);
                    const double sf = fmax(1.0 / 3.0, alpha);
                    lambda *= sf;
                    nu = 2.0;
                    chi = chi_new;
                    ++acc;
                    __syncthreads();
                    if (threadIdx.x == 0) s.cur ^= 1;
                    // the accepted trial cameras become current: swap the FP32/FP64 copies
                    for (int k = threadIdx.x; k < 12 * D.ncam; k += blockDim.x) {
                        const Real t = camr[k];
                        camr[k] = camr_tr[k];
                        camr_tr[k] = t;
                    }
                    __syncthreads();
                    // keep the non-current buffers equal for cameras (fixed ones never change)
                } else {
                    lambda *= nu;
                    nu *= 2;
                    ++rej;
                }
                ++q;
            } while (rho < 0 && q < A.lm.max_trials);
            iters_done = it + 1;
            if (threadIdx.x == 0) trace[it + 1] = chi;
            if (q == A.lm.max_trials) { term = NAV_BA_TERM_TRIALS_EXHAUSTED; break; }
            if (rho == 0) { term = NAV_BA_TERM_ZERO_GAIN; break; }
            if (!isfinite(lambda)) { term = NAV_BA_TERM_LAMBDA_NONFINITE; break; }
        }
    }
    const int cur = s.cur;
    double chi_final = chi;
    if (mixed && !bad) {
        // the mixed form reports FP64 costs of its initial and final states; its trace holds the
        // FP32-residual costs the damping decisions used
        cams_fp64<Real>(D, s, cur, camd);
        chi_final = window_cost<double, Real>(A, D, s, camd, A.x[cur]);
    }
    for (int c = threadIdx.x; c < D.ncam; c += blockDim.x) A.cam_out[D.cam0 + c] = s.cams[cur][c];
    for (int p = threadIdx.x; p < D.npt; p += blockDim.x) {
        const long long gp = D.pt0 + p;
#pragma unroll
        for (int k = 0; k < 4; ++k) A.pt_out[4 * gp + k] = A.x[cur][4 * gp + k];
    }
    if (threadIdx.x == 0) {
        st->initial_cost = chi0_fp64;
        st->final_cost = chi_final;
        st->final_lambda = lambda;
        st->iterations_done = iters_done;
        st->accepted = acc;
        st->rejected = rej;
        st->termination = term;
        st->status = bad ? NAV_BA_ERR_NONFINITE_COST : NAV_BA_OK;
    }
    __syncthreads();
}

template <class Real>
__global__ void __launch_bounds__(sizeof(Real) == 8 ? 256 : 512) window_lm_kernel(WinArgs<Real> A) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    SmemHead& s = *reinterpret_cast<SmemHead*>(smem_raw);
    Real* camr = reinterpret_cast<Real*>(smem_raw + sizeof(SmemHead));  // [2][kWinMaxCams][12]
    double* camd = reinterpret_cast<double*>(smem_raw + sizeof(SmemHead) + 2 * kWinMaxCams * 12 * sizeof(double));
    double* S = camd + kWinMaxCams * 12;
    double* bs = S + (size_t)A.max_m * A.ld;
    for (;;) {
        if (threadIdx.x == 0) {
            const int k = atomicAdd(A.queue, 1);
            s.win = k < A.n_win ? A.order[k] : -1;
        }
        __syncthreads();
        const int w = s.win;
        __syncthreads();
        if (w < 0) break;
        solve_window<Real>(A, w, s, S, bs, camr, camd);
        if (A.debug) break;
    }
}

size_t window_smem_bytes(int max_m) {
    const int ld = max_m + 1;
    return sizeof(SmemHead) + 3 * kWinMaxCams * 12 * sizeof(double) + (size_t)max_m * ld * sizeof(double) +
           (size_t)max_m * sizeof(double);
}

template <class Real>
cudaError_t launch_typed(PreparedBatch& pb, cudaStream_t stream, int threads, double debug_lambda) {
    WindowBatch& b = pb.dev;
    WinArgs<Real> A;
    A.win = b.d_win;
    A.n_win = b.n_queue;
    A.order = b.d_order;
    A.queue = b.d_queue;
    A.cam_init = b.d_cam_init;
    A.cam_free = b.d_cam_free;
    A.pt_init = b.d_pt_init;
    A.pt_free = b.d_pt_free;
    A.pt_eoff = b.d_pt_eoff;
    A.edge_cam = b.d_edge_cam;
    A.edge_pt = b.d_edge_pt;
    A.edge_uv = b.d_edge_uv;
    A.x[0] = b.d_x[0];
    A.x[1] = b.d_x[1];
    A.pt_vg = (Real*)b.d_pt_vg;
    A.pt_vinv = (Real*)b.d_pt_vinv;
    A.edge_jce = (Real*)b.d_edge_jce;
    A.edge_w = (Real*)b.d_edge_w;
    A.edge_y = (Real*)b.d_edge_y;
    A.cam_list = b.d_cam_list;
    A.cam_out = b.d_cam_out;
    A.pt_out = b.d_pt_out;
    A.trace = b.d_trace;
    A.trace_stride = b.trace_stride;
    A.stats = b.d_stats;
    A.debug = debug_lambda >= 0 ? b.d_debug : nullptr;
    A.debug_lambda = debug_lambda;
    A.intr = pb.intr;
    A.lm = pb.lm;
    A.max_m = b.max_m;
    A.ld = b.max_m + 1;
    const size_t smem = window_smem_bytes(b.max_m);
    cudaError_t err = cudaFuncSetAttribute(window_lm_kernel<Real>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (err != cudaSuccess) return err;
    int dev = 0, nsm = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, window_lm_kernel<Real>, threads, smem);
    if (err != cudaSuccess) return err;
    if (per_sm < 1) return cudaErrorInvalidConfiguration;
    int grid = nsm * per_sm;
    if (grid > b.n_queue) grid = b.n_queue;
    if (debug_lambda >= 0) grid = 1;
    err = cudaMemsetAsync(b.d_queue, 0, sizeof(int32_t), stream);
    if (err != cudaSuccess) return err;
    window_lm_kernel<Real><<<grid, threads, smem, stream>>>(A);
    return cudaGetLastError();
}

}  // namespace

cudaError_t window_batch_launch(PreparedBatch& pb, cudaStream_t stream, int precision, int threads,
                                double debug_lambda) {
    if (pb.dev.n_queue == 0) return cudaSuccess;
    if (precision == NAV_BA_MIXED) return launch_typed<float>(pb, stream, threads, debug_lambda);
    return launch_typed<double>(pb, stream, threads, debug_lambda);
}

// ---- per-observation linearization (parity entry point) ---------------------------------

namespace {

template <class Real>
__global__ void linearize_obs_kernel(int n, const double* pose12, const double* pts, const double* uv,
                                     const int32_t* oc, const int32_t* op, Intr intr, int robust,
                                     double delta, double* e, double* jc, double* jp, double* w) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    CamState cs;
    cam_from_pose12(pose12 + 12LL * oc[k], cs);
    Real cr[12], X[3], z[2];
    cam_real<Real>(cs, cr);
    for (int i = 0; i < 3; ++i) X[i] = (Real)pts[3LL * op[k] + i];
    z[0] = (Real)uv[2LL * k];
    z[1] = (Real)uv[2LL * k + 1];
    EdgeLin<Real> L;
    edge_linearize<Real>(intr, cr, cr + 9, X, z, robust != 0, (Real)delta, L);
    if (e) { e[2LL * k] = L.e[0]; e[2LL * k + 1] = L.e[1]; }
    if (jc) for (int i = 0; i < 12; ++i) jc[12LL * k + i] = L.jc[i];
    if (jp) for (int i = 0; i < 6; ++i) jp[6LL * k + i] = L.jp[i];
    if (w) w[k] = L.w;
}

}  // namespace

cudaError_t linearize_observations(const nav_ba_problem& p, const nav_ba_options& o, cudaStream_t stream,
                                   double* e, double* jc, double* jp, double* w, std::string* why) {
    const int n = p.n_obs;
    if (n == 0) return cudaSuccess;
    double *d_pose = nullptr, *d_pts = nullptr, *d_uv = nullptr, *d_out = nullptr;
    int32_t *d_oc = nullptr, *d_op = nullptr;
    const size_t out_per = 2 + 12 + 6 + 1;
    cudaError_t err = cudaSuccess;
    auto chk = [&](cudaError_t x) {
        if (err == cudaSuccess && x != cudaSuccess) err = x;
    };
    chk(cudaMallocAsync(&d_pose, sizeof(double) * 12 * std::max(1, p.n_cams), stream));
    chk(cudaMallocAsync(&d_pts, sizeof(double) * 3 * std::max(1, p.n_points), stream));
    chk(cudaMallocAsync(&d_uv, sizeof(double) * 2 * n, stream));
    chk(cudaMallocAsync(&d_oc, sizeof(int32_t) * n, stream));
    chk(cudaMallocAsync(&d_op, sizeof(int32_t) * n, stream));
    chk(cudaMallocAsync(&d_out, sizeof(double) * out_per * n, stream));
    if (err == cudaSuccess) {
        chk(cudaMemcpyAsync(d_pose, p.cam_pose, sizeof(double) * 12 * p.n_cams, cudaMemcpyHostToDevice, stream));
        chk(cudaMemcpyAsync(d_pts, p.points, sizeof(double) * 3 * p.n_points, cudaMemcpyHostToDevice, stream));
        chk(cudaMemcpyAsync(d_uv, p.obs_uv, sizeof(double) * 2 * n, cudaMemcpyHostToDevice, stream));
        chk(cudaMemcpyAsync(d_oc, p.obs_cam, sizeof(int32_t) * n, cudaMemcpyHostToDevice, stream));
        chk(cudaMemcpyAsync(d_op, p.obs_point, sizeof(int32_t) * n, cudaMemcpyHostToDevice, stream));
    }
    if (err == cudaSuccess) {
        Intr in{p.intrinsics[0], p.intrinsics[1], p.intrinsics[2], p.intrinsics[3], p.intrinsics[4],
                p.intrinsics[5], p.camera_model};
        double* oe = d_out;
        double* ojc = oe + 2LL * n;
        double* ojp = ojc + 12LL * n;
        double* ow = ojp + 6LL * n;
        const int threads = 128, blocks = (n + threads - 1) / threads;
        if (o.precision == NAV_BA_MIXED)
            linearize_obs_kernel<float><<<blocks, threads, 0, stream>>>(n, d_pose, d_pts, d_uv, d_oc, d_op, in, o.robust,
                                                                        o.huber_delta, oe, ojc, ojp, ow);
        else
            linearize_obs_kernel<double><<<blocks, threads, 0, stream>>>(n, d_pose, d_pts, d_uv, d_oc, d_op, in, o.robust,
                                                                         o.huber_delta, oe, ojc, ojp, ow);
        chk(cudaGetLastError());
        if (e) chk(cudaMemcpyAsync(e, oe, sizeof(double) * 2 * n, cudaMemcpyDeviceToHost, stream));
        if (jc) chk(cudaMemcpyAsync(jc, ojc, sizeof(double) * 12 * n, cudaMemcpyDeviceToHost, stream));
        if (jp) chk(cudaMemcpyAsync(jp, ojp, sizeof(double) * 6 * n, cudaMemcpyDeviceToHost, stream));
        if (w) chk(cudaMemcpyAsync(w, ow, sizeof(double) * n, cudaMemcpyDeviceToHost, stream));
    }
    cudaFreeAsync(d_pose, stream);
    cudaFreeAsync(d_pts, stream);
    cudaFreeAsync(d_uv, stream);
    cudaFreeAsync(d_oc, stream);
    cudaFreeAsync(d_op, stream);
    cudaFreeAsync(d_out, stream);
    chk(cudaStreamSynchronize(stream));
    if (err != cudaSuccess && why) *why = cudaGetErrorString(err);
    return err;
}

// ---- upload / free ------------------------------------------------------------------------

static size_t real_size(int precision) { return precision == NAV_BA_MIXED ? sizeof(float) : sizeof(double); }

void window_batch_free(WindowBatch& b) {
    void* ptrs[] = {b.d_win, b.d_order, b.d_queue, b.d_cam_init, b.d_cam_free, b.d_pt_init, b.d_pt_free,
                    b.d_pt_eoff, b.d_edge_cam, b.d_edge_pt, b.d_edge_uv, b.d_x[0], b.d_x[1], b.d_pt_vg,
                    b.d_pt_vinv, b.d_edge_jce, b.d_edge_w, b.d_edge_y, b.d_cam_list, b.d_cam_out, b.d_pt_out,
                    b.d_trace, b.d_stats, b.d_debug};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    b = WindowBatch();
}

cudaError_t window_batch_upload(PreparedBatch& pb, cudaStream_t stream, int precision, int trace_stride,
                                std::string* why) {
    window_batch_free(pb.dev);
    WindowBatch& b = pb.dev;
    // windows that need the engine (others were resolved on the host)
    std::vector<int32_t> idx;
    for (size_t i = 0; i < pb.host.size(); ++i)
        if (pb.host_status[i] == NAV_BA_OK) idx.push_back((int32_t)i);
    pb.desc.assign(pb.host.size(), WinDesc{});
    int64_t nc = 0, np = 0, ne = 0;
    int max_m = 0, max_nc = 0;
    for (size_t i = 0; i < pb.host.size(); ++i) {
        const HostWindow& h = pb.host[i];
        WinDesc& d = pb.desc[i];
        d.cam0 = (int32_t)nc; d.ncam = h.ncam;
        d.pt0 = (int32_t)np; d.npt = h.npt;
        d.e0 = (int32_t)ne; d.ne = h.ne;
        d.nfc = h.nfc; d.nfp = h.nfp;
        nc += h.ncam; np += h.npt; ne += h.ne;
        if (pb.host_status[i] == NAV_BA_OK) {
            max_m = std::max(max_m, 6 * h.nfc);
            max_nc = std::max(max_nc, h.ncam);
        }
    }
    if (nc > INT32_MAX || np > INT32_MAX || ne > INT32_MAX - 1) {
        if (why) *why = "batch too large for 32-bit indices";
        return cudaErrorInvalidValue;
    }
    b.n_win = (int32_t)pb.host.size();
    b.ncam = nc; b.npt = np; b.ne = ne;
    b.max_m = max_m;
    b.max_ncam = max_nc;
    b.precision = precision;
    b.trace_stride = trace_stride;
    // host staging
    std::vector<CamState> cam(nc);
    std::vector<int32_t> cam_free(nc), pt_free(np), pt_eoff(np + 1), edge_cam(ne), edge_pt(ne);
    std::vector<double> pt(4 * np), uv(2 * ne);
    for (size_t i = 0; i < pb.host.size(); ++i) {
        const HostWindow& h = pb.host[i];
        const WinDesc& d = pb.desc[i];
        std::copy(h.cam.begin(), h.cam.end(), cam.begin() + d.cam0);
        std::copy(h.cam_free.begin(), h.cam_free.end(), cam_free.begin() + d.cam0);
        std::copy(h.pt_free.begin(), h.pt_free.end(), pt_free.begin() + d.pt0);
        std::copy(h.pt.begin(), h.pt.end(), pt.begin() + 4LL * d.pt0);
        for (int k = 0; k < h.npt; ++k) pt_eoff[d.pt0 + k] = d.e0 + h.pt_eoff[k];
        std::copy(h.edge_cam.begin(), h.edge_cam.end(), edge_cam.begin() + d.e0);
        std::copy(h.edge_pt.begin(), h.edge_pt.end(), edge_pt.begin() + d.e0);
        std::copy(h.edge_uv.begin(), h.edge_uv.end(), uv.begin() + 2LL * d.e0);
    }
    pt_eoff[np] = (int32_t)ne;
    // schedule: largest windows first (the most edges), engine windows only
    std::vector<int32_t> order = idx;
    std::stable_sort(order.begin(), order.end(), [&](int32_t x, int32_t y) {
        const double wx = (double)pb.host[x].ne + 50.0 * pb.host[x].nfc * pb.host[x].nfc;
        const double wy = (double)pb.host[y].ne + 50.0 * pb.host[y].nfc * pb.host[y].nfc;
        return wx > wy;
    });
    const size_t rs = real_size(precision);
    cudaError_t err = cudaSuccess;
    auto alloc = [&](auto** p, size_t bytes) {
        if (err != cudaSuccess) return;
        bytes = std::max<size_t>(bytes, 16);
        err = cudaMalloc((void**)p, bytes);
        b.bytes += bytes;
    };
    alloc(&b.d_win, sizeof(WinDesc) * pb.desc.size());
    alloc(&b.d_order, sizeof(int32_t) * order.size());
    alloc(&b.d_queue, sizeof(int32_t));
    alloc(&b.d_cam_init, sizeof(CamState) * nc);
    alloc(&b.d_cam_free, sizeof(int32_t) * nc);
    alloc(&b.d_pt_init, sizeof(double) * 4 * np);
    alloc(&b.d_pt_free, sizeof(int32_t) * np);
    alloc(&b.d_pt_eoff, sizeof(int32_t) * (np + 1));
    alloc(&b.d_edge_cam, sizeof(int32_t) * ne);
    alloc(&b.d_edge_pt, sizeof(int32_t) * ne);
    alloc(&b.d_edge_uv, sizeof(double) * 2 * ne);
    alloc(&b.d_x[0], sizeof(double) * 4 * np);
    alloc(&b.d_x[1], sizeof(double) * 4 * np);
    alloc(&b.d_pt_vg, rs * 12 * np);
    alloc(&b.d_pt_vinv, rs * 8 * np);
    alloc(&b.d_edge_jce, rs * 16 * ne);
    alloc(&b.d_edge_w, rs * 18 * ne);
    alloc(&b.d_edge_y, rs * 18 * ne);
    alloc(&b.d_cam_list, sizeof(int32_t) * ne);
    alloc(&b.d_cam_out, sizeof(CamState) * nc);
    alloc(&b.d_pt_out, sizeof(double) * 4 * np);
    alloc(&b.d_trace, sizeof(double) * trace_stride * pb.desc.size());
    alloc(&b.d_stats, sizeof(WinStats) * pb.desc.size());
    alloc(&b.d_debug, sizeof(double) * ((size_t)max_m * max_m + max_m));
    b.h2d_bytes = 0;
    auto up = [&](void* dst, const void* src, size_t bytes) {
        if (err != cudaSuccess || bytes == 0) return;
        err = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, stream);
        b.h2d_bytes += (int64_t)bytes;
    };
    up(b.d_win, pb.desc.data(), sizeof(WinDesc) * pb.desc.size());
    up(b.d_order, order.data(), sizeof(int32_t) * order.size());
    up(b.d_cam_init, cam.data(), sizeof(CamState) * nc);
    up(b.d_cam_free, cam_free.data(), sizeof(int32_t) * nc);
    up(b.d_pt_init, pt.data(), sizeof(double) * 4 * np);
    up(b.d_pt_free, pt_free.data(), sizeof(int32_t) * np);
    up(b.d_pt_eoff, pt_eoff.data(), sizeof(int32_t) * (np + 1));
    up(b.d_edge_cam, edge_cam.data(), sizeof(int32_t) * ne);
    up(b.d_edge_pt, edge_pt.data(), sizeof(int32_t) * ne);
    up(b.d_edge_uv, uv.data(), sizeof(double) * 2 * ne);
    if (err == cudaSuccess) err = cudaStreamSynchronize(stream);
    b.n_queue = (int32_t)order.size();
    if (err != cudaSuccess && why) *why = cudaGetErrorString(err);
    return err;
}

}  // namespace navba
