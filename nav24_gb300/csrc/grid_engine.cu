// grid_engine.cu - one large BA problem on the whole GPU (problems beyond the window engine's
// 24 free cameras: the 200-camera grid, the 50-camera sphere cap, global BA after map merges).
//
// Every phase of an LM iteration is a grid-wide kernel over all points / edges / cameras; the
// Levenberg-Marquardt control (g2o OptimizationAlgorithmLevenberg::solve semantics, as in the
// window engine) runs on the host, which reads the two reduced scalars of each damping trial
// (cost and dx^T(lambda dx + b)) and decides.  Phases:
//   lin_points    thread per point: e, J, Huber weight, V_p, g_p, W_e (shared with the window engine)
//   lin_cameras   warp per chunk of <= 256 edges of one camera (camera-major list), U/g_c partial
//                 sums reduced per camera in a fixed order (no atomics)
//   schur_points  thread per point: chol(V + lambda I), L, t, A_e = W_e L^T (shared)
//   schur_blocks  warp per nonzero 6x6 block of S over its pair list: S_ab = [a==b](U_a + lambda I)
//                 - sum A_i A_j^T into a dense FP64 S; b'
//   cholesky      one thread-block cluster, right-looking 32x32 tiles inside the envelope of S
//                 (tiles left of a tile row's first nonzero tile stay zero), FP64, one reciprocal
//                 square root per column
//   solve         one CTA, tile-blocked forward/back substitution inside the envelope
//   update        thread per point (dx_p = L^T (t - sum A^T dx_c), shared) and per camera (SE(3))
//   cost          thread per point, per-block partial sums reduced on the host in a fixed order
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>

#include <cooperative_groups.h>

#include "engine.hpp"
#include "lm_device.cuh"

namespace cg = cooperative_groups;

namespace navba {
namespace {

constexpr unsigned kFullG = 0xffffffffu;
constexpr int kTile = 32;
constexpr int kCamChunk = 256;

__device__ __forceinline__ CC grid_view() {
    CC c{};
    c.rank = 0;
    c.csize = 1;
    c.lane = threadIdx.x & 31;
    c.wid = threadIdx.x >> 5;
    c.nw = blockDim.x >> 5;
    c.gt = blockIdx.x * blockDim.x + threadIdx.x;
    c.CT = gridDim.x * blockDim.x;
    c.gw = blockIdx.x * c.nw + c.wid;
    c.CW = gridDim.x * c.nw;
    return c;
}

// Block reduction (sum or max) of one double; thread 0 writes out[blockIdx.x].
template <bool MAX>
__device__ void block_partial(double v, double* out) {
    __shared__ double red[32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const double t = __shfl_down_sync(kFullG, v, o);
        v = MAX ? fmax(v, t) : v + t;
    }
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double r = red[0];
        for (int i = 1; i < (int)(blockDim.x >> 5); ++i) r = MAX ? fmax(r, red[i]) : r + red[i];
        out[blockIdx.x] = r;
    }
}

template <class Cost, class Real>
__global__ void k_cost(WinArgs<Real> A, WinDesc D, const Cost* camc, const double* X, double* part) {
    const CC c = grid_view();
    block_partial<false>(cost_partial<Cost, Real>(A, c, D, camc, X), part);
}

template <class Real>
__global__ void k_lin_points(WinArgs<Real> A, WinDesc D, const Real* camr, const double* X, double* part) {
    const CC c = grid_view();
    block_partial<true>(linearize_points<Real>(A, c, D, camr, X), part);
}

// Camera-major re-linearization: one warp per work item (free camera a, edges [e0, e0 + n) of its
// list); the warp's 27 sums (U packed lower, g_c) go to upart[item].
template <class Real>
__global__ void k_lin_cams(WinArgs<Real> A, const int4* items, int n_items, const int32_t* cam_list, const int32_t* fcam,
                           const Real* camr, const double* X, double* upart) {
    const CC c = grid_view();
    const Real delta = (Real)A.lm.huber_delta;
    for (int it = c.gw; it < n_items; it += c.CW) {
        const int4 w = items[it];  // x: free camera, y: list start, z: count
        const Real* cr = camr + 12 * fcam[w.x];
        Real u[27];
#pragma unroll
        for (int k = 0; k < 27; ++k) u[k] = Real(0);
        for (int i = c.lane; i < w.z; i += 32) {
            const int e = cam_list[w.y + i];
            const int gp = A.edge_pt[e];
            const Real Xr[3] = {(Real)X[4LL * gp], (Real)X[4LL * gp + 1], (Real)X[4LL * gp + 2]};
            const Real z[2] = {(Real)A.edge_uv[2LL * e], (Real)A.edge_uv[2LL * e + 1]};
            EdgeLin<Real> L;
            edge_linearize<Real>(A.intr, cr, cr + 9, Xr, z, A.lm.robust != 0, delta, L);
            const Real wt = L.w;
#pragma unroll
            for (int r = 0; r < 6; ++r)
#pragma unroll
                for (int q = 0; q <= r; ++q) u[tri(r, q)] += wt * (L.jc[r] * L.jc[q] + L.jc[6 + r] * L.jc[6 + q]);
            const Real we0 = -wt * L.e[0], we1 = -wt * L.e[1];
#pragma unroll
            for (int r = 0; r < 6; ++r) u[21 + r] += L.jc[r] * we0 + L.jc[6 + r] * we1;
        }
#pragma unroll
        for (int k = 0; k < 27; ++k)
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) u[k] += __shfl_xor_sync(kFullG, u[k], o);
#pragma unroll
        for (int k = 0; k < 27; ++k)
            if ((k & 31) == c.lane) upart[28LL * it + k] = (double)u[k];
    }
}

// U[a] = sum of the camera's item partials in item order; per-block max |diag U|.
__global__ void k_reduce_cams(const double* upart, const int32_t* item_off, int nfc, double* U, double* part) {
    double mx = 0.0;
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx < nfc * 27) {
        const int a = idx / 27, k = idx % 27;
        double s = 0.0;
        for (int it = item_off[a]; it < item_off[a + 1]; ++it) s += upart[28LL * it + k];
        U[28LL * a + k] = s;
        if (k < 21) {
            // diagonal entries of the packed lower 6x6 are tri(r, r)
            if (k == 0 || k == 2 || k == 5 || k == 9 || k == 14 || k == 20) mx = fabs(s);
        }
    }
    block_partial<true>(mx, part);
}

template <class Real>
__global__ void k_schur_points(WinArgs<Real> A, WinDesc D, double lambda, double* part) {
    const CC c = grid_view();
    block_partial<false>((double)schur_points<Real>(A, c, D, lambda), part);
}

// Warp per nonzero block (a >= b) of S over its pair list; dense row-major S (m x m, lower part).
template <class Real>
__global__ void k_schur_blocks(WinArgs<Real> A, const int2* blocks, const int32_t* boff, int nblk, const int2* pairs,
                               const double* U, double lambda, double* S, int m, double* bs) {
    const CC c = grid_view();
    for (int blk = c.gw; blk < nblk; blk += c.CW) {
        const int a = blocks[blk].x, b = blocks[blk].y;
        const int k0 = boff[blk], k1 = boff[blk + 1];
        Real acc[36];
        Real accb[6];
#pragma unroll
        for (int k = 0; k < 36; ++k) acc[k] = Real(0);
#pragma unroll
        for (int k = 0; k < 6; ++k) accb[k] = Real(0);
        for (int k = k0 + c.lane; k < k1; k += 32) {
            const int2 pr = pairs[k];
            Real ai[18], aj[18];
            Rec<Real>::load18(A.edge_a + (long long)Rec<Real>::kEdge * pr.x, ai);
            Rec<Real>::load18(A.edge_a + (long long)Rec<Real>::kEdge * pr.y, aj);
#pragma unroll
            for (int r = 0; r < 6; ++r)
#pragma unroll
                for (int q = 0; q < 6; ++q)
                    acc[r * 6 + q] += ai[r * 3 + 0] * aj[q * 3 + 0] + ai[r * 3 + 1] * aj[q * 3 + 1] + ai[r * 3 + 2] * aj[q * 3 + 2];
            if (a == b && pr.x == pr.y) {
                const Real* t = A.pt_lt + 12LL * A.edge_pt[pr.x] + 6;
                const Real t0 = t[0], t1 = t[1], t2 = t[2];
#pragma unroll
                for (int r = 0; r < 6; ++r) accb[r] += ai[r * 3 + 0] * t0 + ai[r * 3 + 1] * t1 + ai[r * 3 + 2] * t2;
            }
        }
#pragma unroll
        for (int k = 0; k < 36; ++k)
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) acc[k] += __shfl_xor_sync(kFullG, acc[k], o);
        if (a == b) {
#pragma unroll
            for (int k = 0; k < 6; ++k)
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) accb[k] += __shfl_xor_sync(kFullG, accb[k], o);
        }
#pragma unroll
        for (int k = 0; k < 36; ++k) {
            if ((k & 31) != c.lane) continue;
            const int r = k / 6, q = k % 6;
            if (a == b && q > r) continue;
            double v = -(double)acc[k];
            if (a == b) {
                v += U[28LL * a + tri(r, q)];
                if (r == q) v += lambda;
            }
            S[(size_t)(6 * a + r) * m + 6 * b + q] = v;
        }
        if (a == b && c.lane < 6) {
#pragma unroll
            for (int k = 0; k < 6; ++k)
                if (k == c.lane) bs[6 * a + k] = U[28LL * a + 21 + k] - (double)accb[k];
        }
    }
}

// ---- FP64 tiled Cholesky inside the envelope (one thread-block cluster) ------------------

__device__ __forceinline__ void gsync() { cg::this_cluster().sync(); }

// tfirst[I]: first tile column of tile row I that may be nonzero (the envelope, at tile level).
__global__ void k_cholesky(double* S, int m, const int32_t* tfirst, double* rinv, int32_t* ok) {
    __shared__ double tk[kTile][kTile + 1];
    __shared__ double ta[kTile][kTile + 1];
    __shared__ double tb[kTile][kTile + 1];
    __shared__ double rv[kTile];
    __shared__ int sok;
    cg::cluster_group cl = cg::this_cluster();
    const int rank = (int)cl.block_rank(), cs = (int)cl.num_blocks();
    const int tid = threadIdx.x, nth = blockDim.x;
    const int nt = (m + kTile - 1) / kTile;
    if (tid == 0) sok = 1;
    __syncthreads();
    for (int K = 0; K < nt; ++K) {
        const int k0 = K * kTile, kb = min(kTile, m - k0);
        if (rank == 0) {
            for (int idx = tid; idx < kTile * kTile; idx += nth) {
                const int i = idx / kTile, j = idx % kTile;
                tk[i][j] = (i < kb && j <= i) ? S[(size_t)(k0 + i) * m + k0 + j] : 0.0;
            }
            __syncthreads();
            for (int j = 0; j < kb; ++j) {
                if (tid == 0) {
                    const double d = tk[j][j];
                    double r;
                    if (!(d > 0.0) || !isfinite(d)) {
                        sok = 0;
                        r = 1.0;
                        tk[j][j] = 1.0;
                    } else {
                        r = rsqrt(d);
                        tk[j][j] = d * r;
                    }
                    rv[j] = r;
                    rinv[k0 + j] = r;
                }
                __syncthreads();
                for (int i = j + 1 + tid; i < kb; i += nth) tk[i][j] *= rv[j];
                __syncthreads();
                const int w = kb - j - 1;
                for (int idx = tid; idx < w * w; idx += nth) {
                    const int i = j + 1 + idx / w, l = j + 1 + idx % w;
                    if (l <= i) tk[i][l] -= tk[i][j] * tk[l][j];
                }
                __syncthreads();
            }
            for (int idx = tid; idx < kb * kb; idx += nth) {
                const int i = idx / kb, j = idx % kb;
                if (j <= i) S[(size_t)(k0 + i) * m + k0 + j] = tk[i][j];
            }
            if (tid == 0 && !sok) ok[0] = 0;
        }
        gsync();
        // panel: L_IK = A_IK L_KK^-T for the tile rows below whose envelope reaches column K
        int cnt = 0;
        bool loaded = false;
        for (int I = K + 1; I < nt; ++I) {
            if (tfirst[I] > K) continue;
            if ((cnt++ % cs) != rank) continue;
            if (!loaded) {
                for (int idx = tid; idx < kTile * kTile; idx += nth) {
                    const int i = idx / kTile, j = idx % kTile;
                    tk[i][j] = (i < kb && j <= i) ? S[(size_t)(k0 + i) * m + k0 + j] : 0.0;
                }
                for (int j = tid; j < kb; j += nth) rv[j] = rinv[k0 + j];
                loaded = true;
            }
            const int i0 = I * kTile, ib = min(kTile, m - i0);
            __syncthreads();
            for (int idx = tid; idx < kTile * kTile; idx += nth) {
                const int i = idx / kTile, j = idx % kTile;
                ta[i][j] = (i < ib && j < kb) ? S[(size_t)(i0 + i) * m + k0 + j] : 0.0;
            }
            __syncthreads();
            // forward substitution, row-parallel: x_c = (a_c - sum_{j<c} x_j L_cj) / L_cc
            if (tid < ib) {
                for (int cc = 0; cc < kb; ++cc) {
                    double x = ta[tid][cc];
                    for (int j = 0; j < cc; ++j) x -= ta[tid][j] * tk[cc][j];
                    ta[tid][cc] = x * rv[cc];
                }
            }
            __syncthreads();
            for (int idx = tid; idx < ib * kb; idx += nth) {
                const int i = idx / kb, j = idx % kb;
                S[(size_t)(i0 + i) * m + k0 + j] = ta[i][j];
            }
            __syncthreads();
        }
        gsync();
        // trailing update A_IJ -= L_IK L_JK^T for K < J <= I inside the envelope
        cnt = 0;
        for (int I = K + 1; I < nt; ++I) {
            if (tfirst[I] > K) continue;
            const int i0 = I * kTile, ib = min(kTile, m - i0);
            for (int J = K + 1; J <= I; ++J) {
                if (tfirst[J] > K) continue;
                if ((cnt++ % cs) != rank) continue;
                const int j0 = J * kTile, jb = min(kTile, m - j0);
                __syncthreads();
                for (int idx = tid; idx < kTile * kTile; idx += nth) {
                    const int i = idx / kTile, j = idx % kTile;
                    ta[i][j] = (i < ib && j < kb) ? S[(size_t)(i0 + i) * m + k0 + j] : 0.0;
                    tb[i][j] = (i < jb && j < kb) ? S[(size_t)(j0 + i) * m + k0 + j] : 0.0;
                }
                __syncthreads();
                for (int idx = tid; idx < ib * jb; idx += nth) {
                    const int i = idx / jb, j = idx % jb;
                    if (I == J && j > i) continue;
                    double s = 0.0;
#pragma unroll 8
                    for (int t = 0; t < kTile; ++t) s += ta[i][t] * tb[j][t];
                    S[(size_t)(i0 + i) * m + j0 + j] -= s;
                }
            }
        }
        gsync();
    }
}

// Solve L L^T x = b in place (one CTA), tile-blocked, inside the envelope.
__global__ void k_chol_solve(const double* L, int m, const int32_t* tfirst, const double* rinv, double* x) {
    const int tid = threadIdx.x, nth = blockDim.x, lane = tid & 31;
    const int nt = (m + kTile - 1) / kTile;
    // forward: L y = b
    for (int K = 0; K < nt; ++K) {
        const int k0 = K * kTile, kb = min(kTile, m - k0);
        if (tid < 32) {  // warp 0 solves the diagonal tile
            double v = lane < kb ? x[k0 + lane] : 0.0;
            for (int j = 0; j < kb; ++j) {
                const double xj = __shfl_sync(kFullG, v * (lane == j ? rinv[k0 + j] : 1.0), j);
                if (lane == j) v = xj;
                if (lane > j && lane < kb) v -= L[(size_t)(k0 + lane) * m + k0 + j] * xj;
            }
            if (lane < kb) x[k0 + lane] = v;
        }
        __syncthreads();
        for (int r = k0 + kb + tid; r < m; r += nth) {
            if (tfirst[r / kTile] > K) continue;
            double s = 0.0;
            const double* Lr = L + (size_t)r * m + k0;
            for (int j = 0; j < kb; ++j) s += Lr[j] * x[k0 + j];
            x[r] -= s;
        }
        __syncthreads();
    }
    // backward: L^T x = y
    for (int K = nt - 1; K >= 0; --K) {
        const int k0 = K * kTile, kb = min(kTile, m - k0);
        // x_K -= sum over rows below of L_rK x_r (rows r > tile K whose envelope reaches K)
        for (int j = tid; j < kb; j += nth) {
            double s = 0.0;
            for (int r = k0 + kb; r < m; ++r) {
                if (tfirst[r / kTile] > K) {
                    r = (r / kTile + 1) * kTile - 1;
                    continue;
                }
                s += L[(size_t)r * m + k0 + j] * x[r];
            }
            x[k0 + j] -= s;
        }
        __syncthreads();
        if (tid < 32) {
            double v = lane < kb ? x[k0 + lane] : 0.0;
            for (int j = kb - 1; j >= 0; --j) {
                const double xj = __shfl_sync(kFullG, v * (lane == j ? rinv[k0 + j] : 1.0), j);
                if (lane == j) v = xj;
                if (lane < j) v -= L[(size_t)(k0 + j) * m + k0 + lane] * xj;
            }
            if (lane < kb) x[k0 + lane] = v;
        }
        __syncthreads();
    }
}

// Cameras: trial = exp(dx_a) * current for free cameras; Real / FP64 copies; scale part.
template <class Real>
__global__ void k_update_cams(const CamState* cur, CamState* trial, Real* camr_trial, const int32_t* cam_free, int nc,
                              const double* dc, const double* U, double lambda, double* part) {
    double sc = 0.0;
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < nc) {
        const int a = cam_free[k];
        if (a >= 0) {
            se3_left_update(dc + 6 * a, cur[k], trial[k]);
            for (int r = 0; r < 6; ++r) sc += dc[6 * a + r] * (lambda * dc[6 * a + r] + U[28LL * a + 21 + r]);
        } else {
            trial[k] = cur[k];
        }
        cam_real<Real>(trial[k], camr_trial + 12 * k);
    }
    block_partial<false>(sc, part);
}

template <class Real>
__global__ void k_update_points(WinArgs<Real> A, WinDesc D, double lambda, const double* dc, int cur, double* part) {
    const CC c = grid_view();
    block_partial<false>(update_points<Real>(A, c, D, lambda, dc, cur), part);
}

template <class Real>
__global__ void k_cams_real(const CamState* cams, int nc, Real* out) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < nc) cam_real<Real>(cams[k], out + 12 * k);
}

__global__ void k_init_points(const double* init, double* x0, double* x1, int np4) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < np4) {
        x0[k] = init[k];
        x1[k] = init[k];
    }
}

// ---- host side ---------------------------------------------------------------------------

struct GridHost {
    std::vector<int32_t> cam_list, item_off, fcam, boff, tfirst;
    std::vector<int4> items;
    std::vector<int2> blocks, pairs;
};

void build_grid_host(const HostWindow& h, GridHost& g) {
    const int nfc = h.nfc;
    g.fcam.assign(std::max(1, nfc), 0);
    for (int c = 0; c < h.ncam; ++c)
        if (h.cam_free[c] >= 0) g.fcam[h.cam_free[c]] = c;
    // camera-major list of edges with a free camera (stable: point-major order kept)
    std::vector<int32_t> cnt(nfc + 1, 0);
    for (int e = 0; e < h.ne; ++e) {
        const int a = h.cam_free[h.edge_cam[e]];
        if (a >= 0) cnt[a + 1]++;
    }
    std::vector<int32_t> loff(nfc + 1, 0);
    for (int a = 0; a < nfc; ++a) loff[a + 1] = loff[a] + cnt[a + 1];
    g.cam_list.assign(std::max(1, loff[nfc]), 0);
    std::vector<int32_t> fill(loff.begin(), loff.end() - 1);
    for (int e = 0; e < h.ne; ++e) {
        const int a = h.cam_free[h.edge_cam[e]];
        if (a >= 0) g.cam_list[fill[a]++] = e;
    }
    g.items.clear();
    g.item_off.assign(nfc + 1, 0);
    for (int a = 0; a < nfc; ++a) {
        for (int s = loff[a]; s < loff[a + 1]; s += kCamChunk) g.items.push_back(make_int4(a, s, std::min(kCamChunk, loff[a + 1] - s), 0));
        g.item_off[a + 1] = (int32_t)g.items.size();
    }
    if (g.items.empty()) g.items.push_back(make_int4(0, 0, 0, 0));
    // nonzero lower blocks and their pair lists (per block: pairs in camera-major, point order)
    std::vector<std::vector<int2>> per_block_rows(nfc);
    std::vector<int> mark(nfc, -1);
    std::vector<std::vector<int32_t>> rowcols(nfc);
    for (int i = 0; i < h.npt; ++i) {
        if (h.pt_free[i] < 0) continue;
        for (int e = h.pt_eoff[i]; e < h.pt_eoff[i + 1]; ++e) {
            const int a = h.cam_free[h.edge_cam[e]];
            if (a < 0) continue;
            for (int f = h.pt_eoff[i]; f < h.pt_eoff[i + 1]; ++f) {
                const int b = h.cam_free[h.edge_cam[f]];
                if (b >= 0 && b <= a) rowcols[a].push_back(b);
            }
        }
    }
    std::vector<std::vector<int32_t>> cols(nfc);
    for (int a = 0; a < nfc; ++a) {
        rowcols[a].push_back(a);
        std::sort(rowcols[a].begin(), rowcols[a].end());
        rowcols[a].erase(std::unique(rowcols[a].begin(), rowcols[a].end()), rowcols[a].end());
    }
    // block index of (a, b)
    std::vector<int32_t> row_start(nfc + 1, 0);
    for (int a = 0; a < nfc; ++a) row_start[a + 1] = row_start[a] + (int32_t)rowcols[a].size();
    const int nblk = row_start[nfc];
    g.blocks.resize(std::max(1, nblk));
    for (int a = 0; a < nfc; ++a)
        for (size_t k = 0; k < rowcols[a].size(); ++k) g.blocks[row_start[a] + k] = make_int2(a, rowcols[a][k]);
    auto block_of = [&](int a, int b) {
        const auto& rc = rowcols[a];
        return row_start[a] + (int32_t)(std::lower_bound(rc.begin(), rc.end(), b) - rc.begin());
    };
    std::vector<int32_t> pcnt(nblk + 1, 0);
    for (int a = 0; a < nfc; ++a)
        for (int s = loff[a]; s < loff[a + 1]; ++s) {
            const int e = g.cam_list[s];
            const int i = h.edge_pt[e];
            if (h.pt_free[i] < 0) continue;
            for (int f = h.pt_eoff[i]; f < h.pt_eoff[i + 1]; ++f) {
                const int b = h.cam_free[h.edge_cam[f]];
                if (b >= 0 && b <= a) pcnt[block_of(a, b) + 1]++;
            }
        }
    g.boff.assign(nblk + 1, 0);
    for (int k = 0; k < nblk; ++k) g.boff[k + 1] = g.boff[k] + pcnt[k + 1];
    g.pairs.assign(std::max(1, g.boff[nblk]), make_int2(0, 0));
    std::vector<int32_t> pf(g.boff.begin(), g.boff.end() - 1);
    for (int a = 0; a < nfc; ++a)
        for (int s = loff[a]; s < loff[a + 1]; ++s) {
            const int e = g.cam_list[s];
            const int i = h.edge_pt[e];
            if (h.pt_free[i] < 0) continue;
            for (int f = h.pt_eoff[i]; f < h.pt_eoff[i + 1]; ++f) {
                const int b = h.cam_free[h.edge_cam[f]];
                if (b >= 0 && b <= a) g.pairs[pf[block_of(a, b)]++] = make_int2(e, f);
            }
        }
    if (g.boff.size() == 1) g.boff.push_back(0);
    // envelope at tile level: first nonzero tile column of each tile row
    const int m = 6 * nfc;
    const int nt = (m + kTile - 1) / kTile;
    g.tfirst.assign(std::max(1, nt), 0);
    for (int I = 0; I < nt; ++I) {
        int first = I;
        for (int r = I * kTile; r < std::min(m, (I + 1) * kTile); ++r) {
            const int a = r / 6;
            first = std::min(first, (6 * rowcols[a].front()) / kTile);
        }
        g.tfirst[I] = first;
    }
}

// Device buffers of one grid solve (allocated per call; problems here are large, so the
// allocation cost is small against the solve).
struct GridDev {
    std::vector<void*> ptrs;
    cudaError_t err = cudaSuccess;
    template <class T>
    T* alloc(size_t n) {
        if (err != cudaSuccess) return nullptr;
        void* p = nullptr;
        err = cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T));
        if (err == cudaSuccess) ptrs.push_back(p);
        return static_cast<T*>(p);
    }
    ~GridDev() {
        for (void* p : ptrs) cudaFree(p);
    }
};

template <class T>
cudaError_t up(T* d, const std::vector<T>& h, cudaStream_t s) {
    if (h.empty()) return cudaSuccess;
    return cudaMemcpyAsync(d, h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice, s);
}

template <class Real>
cudaError_t grid_solve_typed(const HostWindow& h, const LmOptions& lm, const Intr& intr, cudaStream_t st,
                             int cluster, GridResult& out, double debug_lambda, std::vector<double>* debug_S) {
    GridHost g;
    build_grid_host(h, g);
    const int nc = h.ncam, np = h.npt, ne = h.ne, nfc = h.nfc;
    const int m = 6 * nfc;
    GridDev dv;
    const size_t rec = Rec<Real>::kEdge;
    // inputs
    CamState* d_cams0 = dv.alloc<CamState>(nc);
    CamState* d_cams1 = dv.alloc<CamState>(nc);
    int32_t* d_cam_free = dv.alloc<int32_t>(nc);
    double* d_pinit = dv.alloc<double>(4LL * np);
    int32_t* d_pfree = dv.alloc<int32_t>(np);
    int32_t* d_peoff = dv.alloc<int32_t>(np + 1LL);
    int32_t* d_ecam = dv.alloc<int32_t>(ne);
    int32_t* d_efc = dv.alloc<int32_t>(ne);
    int32_t* d_ept = dv.alloc<int32_t>(ne);
    double* d_uv = dv.alloc<double>(2LL * ne);
    // scratch
    double* d_x0 = dv.alloc<double>(4LL * np);
    double* d_x1 = dv.alloc<double>(4LL * np);
    Real* d_vg = dv.alloc<Real>(12LL * np);
    Real* d_lt = dv.alloc<Real>(12LL * np);
    Real* d_w = dv.alloc<Real>(rec * ne);
    Real* d_a = dv.alloc<Real>(rec * ne);
    Real* d_camr0 = dv.alloc<Real>(12LL * nc);
    Real* d_camr1 = dv.alloc<Real>(12LL * nc);
    double* d_camd = dv.alloc<double>(12LL * nc);
    int32_t* d_list = dv.alloc<int32_t>(g.cam_list.size());
    int4* d_items = dv.alloc<int4>(g.items.size());
    int32_t* d_item_off = dv.alloc<int32_t>(g.item_off.size());
    int32_t* d_fcam = dv.alloc<int32_t>(g.fcam.size());
    double* d_upart = dv.alloc<double>(28 * g.items.size());
    double* d_U = dv.alloc<double>(28LL * std::max(1, nfc));
    int2* d_blocks = dv.alloc<int2>(g.blocks.size());
    int32_t* d_boff = dv.alloc<int32_t>(g.boff.size());
    int2* d_pairs = dv.alloc<int2>(g.pairs.size());
    int32_t* d_tfirst = dv.alloc<int32_t>(g.tfirst.size());
    double* d_S = dv.alloc<double>((size_t)std::max(1, m) * std::max(1, m));
    double* d_bs = dv.alloc<double>(std::max(1, m));
    double* d_rinv = dv.alloc<double>(std::max(1, m));
    int32_t* d_ok = dv.alloc<int32_t>(1);
    const int TB = 256;
    const int nsm_blocks = 152 * 4;
    const int pblocks = std::max(1, std::min(nsm_blocks, (np + TB - 1) / TB));
    const int cblocks = std::max(1, (nc + TB - 1) / TB);
    const int npart = std::max(pblocks, std::max(cblocks, (nfc * 27 + TB - 1) / TB + 1));
    double* d_part = dv.alloc<double>(npart);
    if (dv.err != cudaSuccess) return dv.err;
    std::vector<int32_t> edge_fc(ne);
    for (int e = 0; e < ne; ++e) edge_fc[e] = h.cam_free[h.edge_cam[e]];
    cudaError_t e = cudaSuccess;
    auto chk = [&](cudaError_t x) {
        if (e == cudaSuccess) e = x;
    };
    chk(up(d_cams0, h.cam, st));
    chk(up(d_cams1, h.cam, st));
    chk(up(d_cam_free, h.cam_free, st));
    chk(up(d_pinit, h.pt, st));
    chk(up(d_pfree, h.pt_free, st));
    chk(up(d_peoff, h.pt_eoff, st));
    chk(up(d_ecam, h.edge_cam, st));
    chk(up(d_efc, edge_fc, st));
    chk(up(d_ept, h.edge_pt, st));
    chk(up(d_uv, h.edge_uv, st));
    chk(up(d_list, g.cam_list, st));
    chk(up(d_items, g.items, st));
    chk(up(d_item_off, g.item_off, st));
    chk(up(d_fcam, g.fcam, st));
    chk(up(d_blocks, g.blocks, st));
    chk(up(d_boff, g.boff, st));
    chk(up(d_pairs, g.pairs, st));
    chk(up(d_tfirst, g.tfirst, st));
    if (e != cudaSuccess) return e;

    WinArgs<Real> A{};
    A.pt_free = d_pfree;
    A.pt_eoff = d_peoff;
    A.edge_cam = d_ecam;
    A.edge_fc = d_efc;
    A.edge_pt = d_ept;
    A.edge_uv = d_uv;
    A.x[0] = d_x0;
    A.x[1] = d_x1;
    A.pt_vg = d_vg;
    A.pt_lt = d_lt;
    A.edge_w = d_w;
    A.edge_a = d_a;
    A.intr = intr;
    A.lm = lm;
    WinDesc D{};
    D.cam0 = 0; D.ncam = nc; D.pt0 = 0; D.npt = np; D.e0 = 0; D.ne = ne; D.nfc = nfc; D.nfp = h.nfp;
    CamState* cams[2] = {d_cams0, d_cams1};
    Real* camr[2] = {d_camr0, d_camr1};
    const bool mixed = sizeof(Real) == 4;
    std::vector<double> hpart(npart);
    auto sum_part = [&](int n, bool mx) -> double {
        if (e != cudaSuccess) return 0.0;
        e = cudaMemcpyAsync(hpart.data(), d_part, sizeof(double) * n, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        double s = 0.0;
        for (int k = 0; k < n; ++k) s = mx ? std::max(s, hpart[k]) : s + hpart[k];
        return s;
    };
    auto cost_of = [&](int buf, bool fp64) -> double {
        if (fp64 && mixed) {
            k_cams_real<double><<<cblocks, TB, 0, st>>>(cams[buf], nc, d_camd);
            k_cost<double, Real><<<pblocks, TB, 0, st>>>(A, D, d_camd, A.x[buf], d_part);
        } else {
            k_cost<Real, Real><<<pblocks, TB, 0, st>>>(A, D, camr[buf], A.x[buf], d_part);
        }
        chk(cudaGetLastError());
        return sum_part(pblocks, false);
    };
    k_init_points<<<(4 * np + TB - 1) / TB, TB, 0, st>>>(d_pinit, d_x0, d_x1, 4 * np);
    k_cams_real<Real><<<cblocks, TB, 0, st>>>(d_cams0, nc, d_camr0);
    k_cams_real<Real><<<cblocks, TB, 0, st>>>(d_cams0, nc, d_camr1);
    chk(cudaGetLastError());
    int cur = 0;
    // costs (initial, every trial) are evaluated in FP64 in both forms: they drive the gain ratio
    double chi = cost_of(0, true);
    out.initial_cost = chi;
    out.trace.assign(lm.iterations + 1, 0.0);
    out.trace[0] = chi;
    out.termination = NAV_BA_TERM_ITERATIONS;
    out.iterations_done = out.accepted = out.rejected = 0;
    if (e != cudaSuccess) return e;
    if (!std::isfinite(chi)) {
        out.status = NAV_BA_ERR_NONFINITE_COST;
        return cudaSuccess;
    }
    out.status = NAV_BA_OK;
    if (nfc + h.nfp == 0) out.termination = NAV_BA_TERM_NOTHING_TO_DO;
    double lambda = 0.0, nu = 2.0;
    int cl = std::max(1, std::min(8, cluster));
    for (int it = 0; out.termination == NAV_BA_TERM_ITERATIONS && it < lm.iterations; ++it) {
        k_lin_points<Real><<<pblocks, TB, 0, st>>>(A, D, camr[cur], A.x[cur], d_part);
        const double mxp = sum_part(pblocks, true);
        if (nfc > 0) {
            const int ni = (int)g.items.size();
            k_lin_cams<Real><<<std::max(1, std::min(nsm_blocks, (ni * 32 + TB - 1) / TB)), TB, 0, st>>>(
                A, d_items, ni, d_list, d_fcam, camr[cur], A.x[cur], d_upart);
            const int rb = (nfc * 27 + TB - 1) / TB;
            k_reduce_cams<<<rb, TB, 0, st>>>(d_upart, d_item_off, nfc, d_U, d_part);
            chk(cudaGetLastError());
        }
        const double mxc = nfc > 0 ? sum_part((nfc * 27 + TB - 1) / TB, true) : 0.0;
        if (e != cudaSuccess) return e;
        if (it == 0) {
            lambda = lm.initial_lambda > 0 ? lm.initial_lambda : lm.tau * std::max(mxp, mxc);
            nu = 2.0;
        }
        double rho = 0.0;
        int q = 0;
        do {
            const double lam_use = (debug_S && it == 0 && q == 0) ? debug_lambda : lambda;
            k_schur_points<Real><<<pblocks, TB, 0, st>>>(A, D, lam_use, d_part);
            const double npd = sum_part(pblocks, false);
            bool ok = npd == 0.0;
            if (nfc > 0) {
                chk(cudaMemsetAsync(d_S, 0, sizeof(double) * (size_t)m * m, st));
                const int nb = (int)g.blocks.size();
                k_schur_blocks<Real><<<std::max(1, std::min(nsm_blocks, (nb * 32 + TB - 1) / TB)), TB, 0, st>>>(
                    A, d_blocks, d_boff, (int)(g.boff.size() - 1), d_pairs, d_U, lam_use, d_S, m, d_bs);
                chk(cudaGetLastError());
                if (debug_S) {
                    debug_S->assign((size_t)m * m + m, 0.0);
                    chk(cudaMemcpyAsync(debug_S->data(), d_S, sizeof(double) * m * m, cudaMemcpyDeviceToHost, st));
                    chk(cudaMemcpyAsync(debug_S->data() + (size_t)m * m, d_bs, sizeof(double) * m, cudaMemcpyDeviceToHost, st));
                    chk(cudaStreamSynchronize(st));
                    return e;
                }
                const int32_t one = 1;
                chk(cudaMemcpyAsync(d_ok, &one, sizeof(int32_t), cudaMemcpyHostToDevice, st));
                cudaLaunchConfig_t cfg = {};
                cudaLaunchAttribute attr[1];
                attr[0].id = cudaLaunchAttributeClusterDimension;
                attr[0].val.clusterDim.x = cl;
                attr[0].val.clusterDim.y = 1;
                attr[0].val.clusterDim.z = 1;
                cfg.attrs = attr;
                cfg.numAttrs = 1;
                cfg.gridDim = dim3(cl);
                cfg.blockDim = dim3(256);
                cfg.stream = st;
                chk(cudaLaunchKernelEx(&cfg, k_cholesky, d_S, m, (const int32_t*)d_tfirst, d_rinv, d_ok));
                int32_t okh = 1;
                chk(cudaMemcpyAsync(&okh, d_ok, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
                chk(cudaStreamSynchronize(st));
                if (e != cudaSuccess) return e;
                ok = ok && okh != 0;
                if (ok) {
                    k_chol_solve<<<1, 256, 0, st>>>(d_S, m, d_tfirst, d_rinv, d_bs);
                } else {
                    chk(cudaMemsetAsync(d_bs, 0, sizeof(double) * m, st));
                }
                chk(cudaGetLastError());
            }
            k_update_cams<Real><<<cblocks, TB, 0, st>>>(cams[cur], cams[cur ^ 1], camr[cur ^ 1], d_cam_free, nc, d_bs, d_U,
                                                         lambda, d_part);
            double scale = sum_part(cblocks, false);
            k_update_points<Real><<<pblocks, TB, 0, st>>>(A, D, lambda, d_bs, cur, d_part);
            scale += sum_part(pblocks, false);
            double chi_new = cost_of(cur ^ 1, true);
            if (e != cudaSuccess) return e;
            if (!ok) chi_new = DBL_MAX;
            rho = chi - chi_new;
            scale += 1e-3;
            rho /= scale;
            if (rho > 0 && std::isfinite(chi_new)) {
                double alpha = 1.0 - std::pow(2 * rho - 1, 3.0);
                alpha = std::min(alpha, 2.0 / 3.0);
                lambda *= std::max(1.0 / 3.0, alpha);
                nu = 2.0;
                chi = chi_new;
                ++out.accepted;
                cur ^= 1;
            } else {
                lambda *= nu;
                nu *= 2;
                ++out.rejected;
            }
            ++q;
        } while (rho < 0 && q < lm.max_trials);
        out.iterations_done = it + 1;
        out.trace[it + 1] = chi;
        if (q == lm.max_trials) out.termination = NAV_BA_TERM_TRIALS_EXHAUSTED;
        else if (rho == 0) out.termination = NAV_BA_TERM_ZERO_GAIN;
        else if (!std::isfinite(lambda)) out.termination = NAV_BA_TERM_LAMBDA_NONFINITE;
        if (out.termination != NAV_BA_TERM_ITERATIONS) break;
    }
    if (out.termination == NAV_BA_TERM_ITERATIONS && out.iterations_done < lm.iterations) out.termination = NAV_BA_TERM_ITERATIONS;
    out.final_cost = chi;
    out.final_lambda = lambda;
    out.trace.resize(out.iterations_done + 1);
    out.cams.resize(nc);
    out.points.resize(4LL * np);
    chk(cudaMemcpyAsync(out.cams.data(), cams[cur], sizeof(CamState) * nc, cudaMemcpyDeviceToHost, st));
    chk(cudaMemcpyAsync(out.points.data(), A.x[cur], sizeof(double) * 4 * np, cudaMemcpyDeviceToHost, st));
    chk(cudaStreamSynchronize(st));
    return e;
}

}  // namespace

cudaError_t grid_solve(const HostWindow& h, const LmOptions& lm, const Intr& intr, int precision, cudaStream_t stream,
                       int cluster, GridResult& out, double debug_lambda, std::vector<double>* debug_S) {
    if (precision == NAV_BA_MIXED)
        return grid_solve_typed<float>(h, lm, intr, stream, cluster, out, debug_lambda, debug_S);
    return grid_solve_typed<double>(h, lm, intr, stream, cluster, out, debug_lambda, debug_S);
}

}  // namespace navba
