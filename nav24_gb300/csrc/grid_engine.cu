// grid_engine.cu - one large BA problem on the whole GPU (problems beyond the window engine's
// 24 free cameras: the 200-camera grid, the 50-camera sphere cap, global BA after map merges, and
// every PCG solve).
//
// Every phase of an LM iteration is a grid-wide kernel over all points / edges / cameras; the
// Levenberg-Marquardt control (g2o OptimizationAlgorithmLevenberg::solve semantics, as in the
// window engine) runs on the host, which reads the reduced scalars of each damping trial
// (cost and dx^T(lambda dx + b)) and decides.  Phases:
//   lin_points    thread per point: e, J, Huber weight, V_p, g_p (shared with the window engine)
//   lin_cameras   warp per chunk of <= 256 edges of one camera (camera-major list), U/g_c partial
//                 sums reduced per camera in a fixed order (no atomics)
//   schur_points  thread per point: chol(V + lambda I), L, t, A_e = W_e L^T with W_e recomputed (shared)
//   schur_blocks  warp per work item (<= 256 observation pairs of one nonzero 6x6 block of S, taken in
//                 order from a counter): S_ab = [a==b](U_a + lambda I) - sum A_i A_j^T, into a dense
//                 FP64 S (Cholesky; the mixed form also its FP32 lower part and the upper mirror) or
//                 block rows of both triangles (explicit PCG); b'
//   cholesky      cooperative persistent kernel, right-looking 32x32 tiles inside the envelope of S
//                 (tiles left of a tile row's first nonzero tile stay zero); FP32 factor + one FP64
//                 refinement in the mixed form; leaves the diagonal tiles' inverses and contiguous
//                 copies of the panel tiles for the solves
//   solve         one CTA, tile by tile inside the envelope, each tile step's data copied ahead into
//                 a shared-memory ring (cp.async); the mixed form's roundings to and from FP32 at
//                 its start and end
//   pcg           cooperative persistent kernel per damped system, block-Jacobi preconditioner:
//                 explicit S (two grid phases per CG iteration) or, for long pair lists, products
//                 through the per-edge records (five phases)
//   update        thread per point (dx_p = L^T (t - sum A^T dx_c), shared) and per camera (SE(3),
//                 warp-sized blocks)
//   cost          thread per edge, per-block partial sums reduced on the host in a fixed order
// With a GridVjp, the accepted steps' states and damping are taped (or a given damping schedule
// is replayed) and the backward pass of vjp_device.cuh runs over the taped steps, last first.
#include <algorithm>
#include <cfloat>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cmath>
#include <cstring>
#include <functional>
#include <memory>
#include <thread>
#include <type_traits>

#include <cooperative_groups.h>

#include "engine.hpp"
#include "lm_device.cuh"
#include "vjp_device.cuh"

namespace cg = cooperative_groups;

namespace navba {
namespace {

constexpr unsigned kFullG = 0xffffffffu;
constexpr int kTile = 32;
// the dynamic shared memory of a triangular solve (x and its ring of tile steps), beside ~2-4 KB
// of static shared memory
constexpr size_t kSolveSmem = 200 * 1024;
constexpr int kCamChunk = 256;
constexpr int kPairChunk = 256;  // pairs per work item of the Schur-block kernel

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

// Block reduction (sum or max) of one double; thread 0 writes out[blockIdx.x] (out[slot] when
// slot >= 0).
template <bool MAX>
__device__ void block_partial(double v, double* out, int slot = -1) {
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
        out[slot >= 0 ? slot : (int)blockIdx.x] = r;
    }
}

// Robust chi2 partial sums; e_out != null: every edge's residual is also stored (rounded to Real).
// Thread per edge (grid-stride over the point-major edges, the point from edge_pt): with a thread
// per point a warp ran as many rounds as its most-observed point, and in the FP64 cost every round
// costs an FP64 instruction per warp whatever its active lanes.  The grid is fixed per problem, so
// the per-thread sums (and the fixed-order block partials) repeat bitwise.
template <class Cost, class Real>
__global__ void k_cost(WinArgs<Real> A, WinDesc D, const Cost* camc, const double* X, double* part,
                       Real* e_out = nullptr) {
    const CC c = grid_view();
    double acc = 0.0;
    const Cost delta = (Cost)A.lm.huber_delta;
    for (int k = c.gt; k < D.ne; k += c.CT) {
        const int e = D.e0 + k, gp = D.pt0 + A.edge_pt[e];
        const Cost Xr[3] = {(Cost)X[4LL * gp], (Cost)X[4LL * gp + 1], (Cost)X[4LL * gp + 2]};
        Cost cr[12];
        cam_load(camc + 12 * A.edge_cam[e], cr);
        const Cost z[2] = {(Cost)A.edge_uv[2LL * e], (Cost)A.edge_uv[2LL * e + 1]};
        if (e_out) {
            Cost Xc[3], uv[2];
            transform(cr, cr + 9, Xr, Xc);
            project<Cost>(A.intr, Xc, uv, nullptr);
            const Cost e0 = z[0] - uv[0], e1v = z[1] - uv[1];
            double rho;
            Cost w;
            huber<Cost>(e0 * e0 + e1v * e1v, A.lm.robust != 0, delta, rho, w);
            acc += rho;
            e_out[2LL * e] = (Real)e0;
            e_out[2LL * e + 1] = (Real)e1v;
        } else {
            acc += edge_cost<Cost>(A.intr, cr, cr + 9, Xr, z, A.lm.robust != 0, delta);
        }
    }
    block_partial<false>(acc, part);
}

// Active edges whose point is at or behind its camera (Z_c <= 0, FP64), per-block partial counts.
template <class Real>
__global__ void k_depth_count(WinArgs<Real> A, WinDesc D, const CamState* cams, const double* X, double* part) {
    const CC c = grid_view();
    double n = 0.0;
    for (int p = c.gt; p < D.npt; p += c.CT) {
        const int gp = D.pt0 + p;
        const double Xp[3] = {X[4LL * gp], X[4LL * gp + 1], X[4LL * gp + 2]};
        const int e1 = A.pt_eoff[gp + 1];
        for (int e = A.pt_eoff[gp]; e < e1; ++e) n += depth_nonpositive(cams[A.edge_cam[e]], Xp) ? 1.0 : 0.0;
    }
    block_partial<false>(n, part);
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
            edge_linearize_e<Real>(A, e, cr, Xr, z, delta, L);
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
        const Real uk = lane_value<27>(u, c.lane);  // one FP64 conversion per warp, not per value
        if (c.lane < 27) upart[28LL * it + c.lane] = (double)uk;
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
__global__ void k_schur_points(WinArgs<Real> A, WinDesc D, double lambda, const Real* camr, const double* X, double* part) {
    const CC c = grid_view();
    block_partial<false>((double)schur_points<Real>(A, c, D, lambda, camr, X), part);
}

// Warp per work item: up to kPairChunk pairs of one nonzero block (a >= b) of S.  Output: dense
// row-major S (m x m, lower part; with S32 also mirrored into the upper part, and the lower part
// rounded to FP32 into S32, the mixed form's factorization input), or, with Sb, block rows of both
// triangles in Real (row-major 6x6 per slot; bslot[blk]: the slot of the block and of its
// transpose, -1 on the diagonal, whose block is written whole).  Warps take the items in order from a counter (next, zero at launch), so the
// records being read stay within a window of consecutive camera rows, which stays in L2; items are
// short so that no warp lags far behind the window (a diagonal block holds all of its camera's
// observations).  A block of several items is finished by whichever of its items ends last (count
// in done[blk], zero at launch): it sums the items' partials (48 Real per item in part) in item
// order.  Every sum has a fixed order whichever warps take the items.
template <class Real>
__global__ void k_schur_blocks(WinArgs<Real> A, const int2* blocks, const int32_t* boff, const int4* items,
                               int n_items, const int2* pairs, const double* U, double lambda, double* S, int m,
                               double* bs, Real* Sb, const int2* bslot, int32_t* next, int32_t* done, Real* part,
                               int chunk, float* S32 = nullptr) {
    const CC c = grid_view();
    const int slot = rs36_slot(c.lane);  // this lane's two entries of the block (slot, slot + 1)
    for (;;) {
        int j = 0;
        if (c.lane == 0) j = atomicAdd(next, 1);
        j = __shfl_sync(kFullG, j, 0);
        if (j >= n_items) break;
        const int4 it = items[j];  // block, first and end pair, first item of the block
        const int blk = it.x;
        const int a = blocks[blk].x, b = blocks[blk].y;
        Real acc[36];
        Real accb[6];
#pragma unroll
        for (int k = 0; k < 36; ++k) acc[k] = Real(0);
#pragma unroll
        for (int k = 0; k < 6; ++k) accb[k] = Real(0);
        for (int k = it.y + c.lane; k < it.z; k += 32) {
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
        Real sums[2];
        reduce_scatter36(acc, c.lane, sums[0], sums[1]);  // lane: the two entries it writes
        Real bk = Real(0);
        if (a == b) {
#pragma unroll
            for (int k = 0; k < 6; ++k)
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) accb[k] += __shfl_xor_sync(kFullG, accb[k], o);
            bk = lane_value<6>(accb, c.lane);
        }
        const int np_blk = boff[blk + 1] - boff[blk];
        const int nit = np_blk > chunk ? (int)(((long long)np_blk + chunk - 1) / chunk) : 1;
        double sumd[2] = {(double)sums[0], (double)sums[1]}, bkd = (double)bk;
        if (nit > 1) {
            Real* pp = part + 48LL * j;
#pragma unroll
            for (int rnd = 0; rnd < 2; ++rnd)
                if (slot + rnd < 36) pp[slot + rnd] = sums[rnd];
            if (c.lane < 6) pp[36 + c.lane] = bk;
            __threadfence();
            // every lane's partials and fence come before lane 0 publishes the item as done
            __syncwarp();
            int last = 0;
            if (c.lane == 0) last = atomicAdd(done + blk, 1) == nit - 1;
            if (!__shfl_sync(kFullG, last, 0)) continue;
            __threadfence();
            // the partials are summed in FP64: a diagonal block's sum nearly cancels U_a, and the
            // mixed form factors S in FP32
            const Real* p0 = part + 48LL * it.w;
#pragma unroll
            for (int rnd = 0; rnd < 2; ++rnd) {
                double v = 0.0;
                if (slot + rnd < 36)
                    for (int i = 0; i < nit; ++i) v += (double)__ldcg(p0 + 48LL * i + slot + rnd);
                sumd[rnd] = v;
            }
            double vb = 0.0;
            if (c.lane < 6)
                for (int i = 0; i < nit; ++i) vb += (double)__ldcg(p0 + 48LL * i + 36 + c.lane);
            bkd = vb;
        }
        // one FP64 warp instruction per operation with all lanes active (charged per warp instruction)
        const int2 bs2 = Sb ? bslot[blk] : make_int2(0, -1);
#pragma unroll
        for (int rnd = 0; rnd < 2; ++rnd) {
            const int k = slot + rnd;
            const int r = k / 6, q = k % 6;
            if (k < 36 && (Sb || !(a == b && q > r))) {
                double v = -sumd[rnd];
                if (a == b) {
                    v += U[28LL * a + (r >= q ? tri(r, q) : tri(q, r))];
                    if (r == q) v += lambda;
                }
                if (Sb) {
                    Sb[36LL * bs2.x + k] = (Real)v;
                    if (bs2.y >= 0) Sb[36LL * bs2.y + q * 6 + r] = (Real)v;
                } else {
                    S[(size_t)(6 * a + r) * m + 6 * b + q] = v;
                    if (S32) {
                        S32[(size_t)(6 * a + r) * m + 6 * b + q] = (float)v;
                        if (a != b || q != r) S[(size_t)(6 * b + q) * m + 6 * a + r] = v;
                    }
                }
            }
        }
        if (a == b && c.lane < 6) bs[6 * a + c.lane] = U[28LL * a + 21 + c.lane] - bkd;
    }
}

// ---- Tiled Cholesky inside the envelope -------------------------------------------------

// tfirst[I]: first tile column of tile row I that may be nonzero (the envelope, at tile level);
// rows(K) = the tile rows I > K with tfirst[I] <= K (the panel of tile column K).
//
// Right-looking Cholesky of the envelope over the whole GPU (cooperative launch, every block
// resident).  Per tile column K, every block owning a panel tile of column K factors the diagonal
// tile in its shared memory (warp 0, the tile's rows in lane registers) and solves its panel tiles
// L_IK = A_IK L_KK^-T (warp 0, a row per lane); block 0 also stores L_KK and 1/L_jj once no block
// reads A_KK any more.  The trailing tiles (I, J), I >= J, both in rows(K), are updated
// A_IJ -= L_IK L_JK^T in quarter-tile work items spread over the blocks, first to the blocks
// without panel work.
// - FP64: a grid synchronization after the panels and one after the trailing update.
// - FP32 (latency-bound): one grid synchronization per column.  Phase K applies column K - 1's
//   update to the trailing tiles right of column K while column K is finished: the panel blocks
//   apply it to A_KK and their own panel tiles in shared memory before factoring and solving.
// Either way the updates reach every element column by column.  A non-positive pivot is replaced by 1 and reported through
// fail (set to 1; zero at launch).  Each panel tile is also stored contiguously, transposed into LT and as is into LN (32 x 32
// per entry of the panel list, in list order), and each diagonal tile's inverse into DI (L^-T and
// L^-1, 32 x 32 each, by tile), which the solves read.  Requires 256 threads per block.  tr_ij lists each
// column's trailing tiles by column J
// (J ascending), so the tiles of column K + 1 are the first tr_skip[K] of column K's list.
template <class T>
using TileT = T[kTile][kTile + 1];

// rows r0.. (rb of them) and columns c0.. (cb) of row-major S (leading dimension m) into t; zero
// elsewhere (lower_only: only j <= i)
template <class T>
__device__ __forceinline__ void tile_load(TileT<T>& t, const T* S, int m, int r0, int rb, int c0, int cb,
                                          bool lower_only = false) {
    for (int idx = threadIdx.x; idx < kTile * kTile; idx += blockDim.x) {
        const int i = idx >> 5, j = idx & 31;
        t[i][j] = (i < rb && j < cb && (!lower_only || j <= i)) ? S[(size_t)(r0 + i) * m + c0 + j] : T(0);
    }
}

// s[q] = sum_t a[r + 8q][t] b[c][t] (t = 0..31 in order) for this thread's column c = tid & 31 and
// rows r + 8q, r = tid >> 5 (256 threads: one 32 x 32 tile product)
template <class T>
__device__ __forceinline__ void tile_abt(const TileT<T>& a, const TileT<T>& b, T s[4]) {
    const int c = threadIdx.x & 31, r = threadIdx.x >> 5;
    s[0] = s[1] = s[2] = s[3] = T(0);
#pragma unroll 8
    for (int t = 0; t < kTile; ++t) {
        const T bv = b[c][t];
#pragma unroll
        for (int q = 0; q < 4; ++q) s[q] += a[r + 8 * q][t] * bv;
    }
}

// LL^T of the kb x kb lower tile tk in place; rv[j] receives 1/L_jj.  Per column: the pivot, the
// column scaled by 1/L_jj, the rank-1 update of the columns to its right.  Called by every thread
// of the block; a barrier must follow.
// - FP32: warp 0 alone, lane i holding row i in registers, in panels of 8 columns.  Each column's
//   unscaled values go through shared memory (col, double-buffered): every lane reads the pivot
//   u_cc, forms r = 1/sqrt(u_cc) itself and its L_ic = u_ic r, and updates the panel's columns,
//   u_ij -= (L_ic r) u_jc; one warp barrier per column (a shuffle per element was 5x slower).  The
//   panel's L columns (pcol) then update the columns to its right in one rank-8 pass, so the
//   column-by-column chain touches 8 columns instead of up to 31.
// - FP64: the whole block (warp per row of the update), so that the FP64 products are spread over
//   the SM's four partitions.
constexpr int kDiagPanel = 8;  // FP32 diagonal-tile factorization: columns per panel
template <class T>
__device__ void factor_diag_tile(TileT<T>& tk, T* rv, T (*col)[kTile], T (*pcol)[kTile], int kb, int& bad) {
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    if constexpr (sizeof(T) == 4) {
        if (wid != 0) return;
        T d[kTile];
#pragma unroll
        for (int j = 0; j < kTile; ++j) d[j] = (lane < kb && j <= lane) ? tk[lane][j] : T(0);
        col[0][lane] = d[0];
        __syncwarp();
#pragma unroll
        for (int c0 = 0; c0 < kTile; c0 += kDiagPanel) {
            // the panel's columns one by one, updating only the panel's own columns
#pragma unroll
            for (int cc = c0; cc < c0 + kDiagPanel; ++cc) {
                if (cc < kb) {
                    const T* cu = col[cc & 1];  // column cc, unscaled
                    const T piv = cu[cc];
                    const bool colbad = !(piv > T(0)) || !isfinite(piv);
                    const T r = colbad ? T(1) : rsqrtf(piv);
                    if (colbad) bad = 1;
                    const T li = lane == cc ? (colbad ? T(1) : piv * r) : d[cc] * r;
                    d[cc] = li;
                    pcol[cc - c0][lane] = li;
                    const T wi = li * r;
                    if (lane == 0) rv[cc] = r;
#pragma unroll
                    for (int j = cc + 1; j < c0 + kDiagPanel; ++j)
                        if (lane >= j) d[j] -= wi * cu[j];
                    if (cc + 1 < c0 + kDiagPanel) col[(cc + 1) & 1][lane] = d[cc + 1];
                    __syncwarp();
                }
            }
            // the panel's rank-kDiagPanel update of the columns to its right: u_ij -= sum_c L_ic L_jc
            if (c0 + kDiagPanel < kb) {
#pragma unroll
                for (int j = c0 + kDiagPanel; j < kTile; ++j) {
                    T s = T(0);
#pragma unroll
                    for (int c = 0; c < kDiagPanel; ++c) s += d[c0 + c] * pcol[c][j];
                    if (lane >= j) d[j] -= s;
                }
                col[(c0 + kDiagPanel) & 1][lane] = d[c0 + kDiagPanel];
                __syncwarp();
            }
        }
#pragma unroll
        for (int j = 0; j < kTile; ++j)
            if (lane < kb && j <= lane) tk[lane][j] = d[j];
    } else {
        const int nw = blockDim.x >> 5;
        for (int j = 0; j < kb; ++j) {
            if (tid == 0) {
                const T dj = tk[j][j];
                T r;
                if (!(dj > T(0)) || !isfinite(dj)) {
                    bad = 1;
                    r = T(1);
                    tk[j][j] = T(1);
                } else {
                    r = rsqrt(dj);
                    tk[j][j] = dj * r;
                }
                rv[j] = r;
            }
            __syncthreads();
            for (int i = j + 1 + tid; i < kb; i += blockDim.x) tk[i][j] *= rv[j];
            __syncthreads();
            for (int i = j + 1 + wid; i < kb; i += nw)
                for (int l = j + 1 + lane; l <= i; l += 32) tk[i][l] -= tk[i][j] * tk[l][j];
            __syncthreads();
        }
    }
}

// The inverse of the lower tile L = tk (1/L_jj in rv) by warp 0: lane j forms column j,
// y_i = -(1/L_ii) sum_{j<=k<i} L_ik y_k (y_j = 1/L_jj), and stores it into di (two 32 x 32
// row-major blocks: L^-T, then L^-1), so the triangular solves apply each diagonal tile as a
// product, reading row c of the block for every c with lanes over its columns in both directions.
template <class T>
__device__ void invert_diag_tile(const TileT<T>& tk, const T* rv, T* di) {
    const int lane = threadIdx.x & 31;
    T y[kTile];
#pragma unroll
    for (int i = 0; i < kTile; ++i) {
        T s = T(0);
#pragma unroll
        for (int k = 0; k < i; ++k) s += tk[i][k] * y[k];
        y[i] = i < lane ? T(0) : (i == lane ? rv[i] : -rv[i] * s);
    }
#pragma unroll
    for (int i = 0; i < kTile; ++i) {
        di[lane * kTile + i] = y[i];                  // (L^-T)_lane,i = (L^-1)_i,lane
        di[kTile * kTile + i * kTile + lane] = y[i];  // (L^-1)_i,lane
    }
}

// x L_KK^T = a for the ib rows of ta by warp 0 (lane i: row i in registers):
// x_c = (a_c - sum_{j<c} x_j L_cj) / L_cc, the sum in four partial sums (j mod 4).
template <class T>
__device__ void panel_solve(TileT<T>& ta, const TileT<T>& tk, const T* rv, int ib, int kb) {
    const int lane = threadIdx.x & 31;
    T a[kTile];
#pragma unroll
    for (int j = 0; j < kTile; ++j) a[j] = ta[lane][j];
#pragma unroll
    for (int cc = 0; cc < kTile; ++cc) {
        if (cc < kb) {
            T s0 = T(0), s1 = T(0), s2 = T(0), s3 = T(0);
            int j = 0;
#pragma unroll
            for (; j + 3 < cc; j += 4) {
                s0 += a[j] * tk[cc][j];
                s1 += a[j + 1] * tk[cc][j + 1];
                s2 += a[j + 2] * tk[cc][j + 2];
                s3 += a[j + 3] * tk[cc][j + 3];
            }
#pragma unroll
            for (; j < cc; ++j) s0 += a[j] * tk[cc][j];
            a[cc] = (a[cc] - ((s0 + s1) + (s2 + s3))) * rv[cc];
        }
    }
    if (lane < ib)
#pragma unroll
        for (int j = 0; j < kTile; ++j) ta[lane][j] = a[j];
}

template <class T>
__global__ void __launch_bounds__(256) k_cholesky_coop(T* S, int m, const int32_t* tfirst, const int32_t* pan_off,
                                                       const int32_t* pan_row, const int32_t* tr_off, const int32_t* tr_skip,
                                                       const int2* tr_ij, T* rinv, T* LT, T* LN, T* DI, int32_t* fail,
                                                       unsigned long long* phase) {
    constexpr bool one_sync = sizeof(T) == 4;
    cg::grid_group grid = cg::this_grid();
    __shared__ TileT<T> tk, ta, tb, tc;
    __shared__ T rv[kTile], col[2][kTile], pcol[kDiagPanel][kTile];
    __shared__ int sbad;
    const int tid = threadIdx.x, nb = gridDim.x, bid = blockIdx.x, wid = tid >> 5;
    const int nt = (m + kTile - 1) / kTile;
    // phase timer (block 0's view), accumulated in registers and written once at the end, so the
    // marks add no memory round trip to the chain they measure
    const bool timed = phase && bid == 0 && tid == 0;
    long long tmark = timed ? clock64() : 0;
    unsigned long long tacc[5] = {0, 0, 0, 0, 0};
    auto mark = [&](int k) {
        if (timed) {
            const long long now = clock64();
            tacc[k] += (unsigned long long)(now - tmark);
            tmark = now;
        }
    };
    if (tid == 0) sbad = 0;
    int bad = 0;  // pivot failures this thread saw
    auto store_diag = [&](int k0, int kb) {  // L_KK (from tk) and 1/L_jj into S and rinv
        for (int idx = tid; idx < kb * kb; idx += blockDim.x) {
            const int i = idx / kb, j = idx % kb;
            if (j <= i) S[(size_t)(k0 + i) * m + k0 + j] = tk[i][j];
        }
        for (int j = tid; j < kb; j += blockDim.x) rinv[k0 + j] = rv[j];
    };
    // tk -= a a^T (a: a 32 x 32 tile in shared memory); a barrier follows
    auto sub_aat = [&](TileT<T>& dst, const TileT<T>& a, const TileT<T>& b) {
        T s[4];
        tile_abt(a, b, s);
        const int c = tid & 31, r = tid >> 5;
#pragma unroll
        for (int q = 0; q < 4; ++q) dst[r + 8 * q][c] -= s[q];
    };
    // dst -= a b^T by warps 1..7 (while warp 0 factors the diagonal tile), four partial sums
    auto sub_abt_w = [&](TileT<T>& dst, const TileT<T>& a, const TileT<T>& b) {
        for (int o = tid - kTile; o < kTile * kTile; o += blockDim.x - kTile) {
            const int r = o >> 5, c = o & 31;
            T s4[4] = {T(0), T(0), T(0), T(0)};
#pragma unroll
            for (int t = 0; t < kTile; ++t) s4[t & 3] += a[r][t] * b[c][t];
            dst[r][c] -= (s4[0] + s4[1]) + (s4[2] + s4[3]);
        }
    };
    // panel tile pi of column K: its loads into ta (and L_I,K-1 into tc when it gets column K - 1's
    // update, upd_prev: L_K,K-1 in tb); returns whether it does
    auto panel_load = [&](int K, int pi, bool upd_prev) {
        const int k0 = K * kTile, kb = min(kTile, m - k0), kp = k0 - kTile;
        const int I = pan_row[pan_off[K] + pi], i0 = I * kTile, ib = min(kTile, m - i0);
        const bool upd = upd_prev && tfirst[I] <= K - 1;
        tile_load(ta, S, m, i0, ib, k0, kb);
        if (upd) tile_load(tc, S, m, i0, ib, kp, kTile);
        return upd;
    };
    // panel tile pi of column K, updated, in ta: L_IK = A_IK L_KK^-T (L_KK in tk, 1/L_jj in rv),
    // stored into S and, contiguous, into LT (transposed) and LN for the solves
    auto panel_finish = [&](int K, int pi) {
        const int k0 = K * kTile, kb = min(kTile, m - k0), p0 = pan_off[K];
        const int i0 = pan_row[p0 + pi] * kTile, ib = min(kTile, m - i0);
        if (wid == 0) panel_solve(ta, tk, rv, ib, kb);
        __syncthreads();
        for (int idx = tid; idx < ib * kb; idx += blockDim.x) {
            const int i = idx / kb, j = idx % kb;
            S[(size_t)(i0 + i) * m + k0 + j] = ta[i][j];
        }
        T* lt = LT + (size_t)(p0 + pi) * (kTile * kTile);
        T* ln = LN + (size_t)(p0 + pi) * (kTile * kTile);
        for (int idx = tid; idx < kTile * kTile; idx += blockDim.x) {
            lt[idx] = ta[idx & 31][idx >> 5];
            ln[idx] = ta[idx >> 5][idx & 31];
        }
        __syncthreads();
    };
    // the diagonal tile of column K (minus column K - 1's update with upd_prev), factored, and this
    // block's panel tiles: the first tile's loads go with the diagonal tile's, and its update runs
    // on warps 1..7 while warp 0 factors (FP32)
    auto column = [&](int K, bool upd_prev) {
        const int k0 = K * kTile, kb = min(kTile, m - k0), kp = k0 - kTile;
        const int npan = pan_off[K + 1] - pan_off[K];
        __syncthreads();
        tile_load(tk, S, m, k0, kb, k0, kb, true);
        if (upd_prev) tile_load(tb, S, m, k0, kb, kp, kTile);
        const bool first = bid < npan;
        const bool upd0 = first && panel_load(K, bid, upd_prev);
        __syncthreads();
        if (upd_prev) {
            sub_aat(tk, tb, tb);
            __syncthreads();
        }
        factor_diag_tile(tk, rv, col, pcol, kb, bad);
        if constexpr (sizeof(T) == 4) {
            if (upd0 && wid > 0) sub_abt_w(ta, tc, tb);
        }
        __syncthreads();
        if constexpr (sizeof(T) != 4) {
            if (upd0) {
                sub_aat(ta, tc, tb);
                __syncthreads();
            }
        }
        mark(0);
        if (first) panel_finish(K, bid);
        for (int pi = bid + nb; pi < npan; pi += nb) {
            const bool upd = panel_load(K, pi, upd_prev);
            __syncthreads();
            if (upd) {
                sub_aat(ta, tc, tb);
                __syncthreads();
            }
            panel_finish(K, pi);
        }
        mark(1);
    };
    // trailing update A_IJ -= L_I,c L_J,c^T over the listed tiles [t0, t1) of column c, in
    // quarter-tile work items (8 rows x 32 columns, one output per thread), first to the blocks
    // after the npan panel owners
    auto trailing = [&](int c, int t0, int t1, int npan) {
        const int c0 = c * kTile, nitems = 4 * (t1 - t0);
        int w = bid - min(npan, nb);
        if (w < 0) w += nb;
        for (; w < nitems; w += nb) {
            const int2 ij = tr_ij[t0 + w / 4];
            const int I = ij.x, J = ij.y, r0 = 8 * (w % 4);
            const int i0 = I * kTile, ib = min(kTile, m - i0), j0 = J * kTile, jb = min(kTile, m - j0);
            if (r0 >= ib) continue;  // uniform per block
            __syncthreads();
            for (int idx = tid; idx < kTile * kTile; idx += blockDim.x) {
                const int i = idx >> 5, j = idx & 31;
                tb[i][j] = i < jb ? S[(size_t)(j0 + i) * m + c0 + j] : T(0);
                if (i < 8) ta[i][j] = r0 + i < ib ? S[(size_t)(i0 + r0 + i) * m + c0 + j] : T(0);
            }
            __syncthreads();
            const int r = tid >> 5, cc = tid & 31;  // 256 threads: 8 rows x 32 columns
            if (r0 + r < ib && cc < jb && !(I == J && cc > r0 + r)) {
                T s4[4] = {T(0), T(0), T(0), T(0)};  // four partial sums (t mod 4)
#pragma unroll
                for (int t = 0; t < kTile; ++t) s4[t & 3] += ta[r][t] * tb[cc][t];
                S[(size_t)(i0 + r0 + r) * m + j0 + cc] -= (s4[0] + s4[1]) + (s4[2] + s4[3]);
            }
        }
    };
    if constexpr (one_sync) {
        for (int K = 0; K < nt; ++K) {
            const int k0 = K * kTile, kb = min(kTile, m - k0);
            const int npan = pan_off[K + 1] - pan_off[K];
            const bool upd_prev = K > 0 && tfirst[K] <= K - 1;  // L_K,K-1 is inside the envelope
            // A_KK minus column K - 1's update, factored by every panel block (redundantly)
            if (bid == 0 || bid < npan) column(K, upd_prev);
            // column K - 1's update of the trailing tiles right of column K
            if (K > 0) trailing(K - 1, tr_off[K - 1] + tr_skip[K - 1], tr_off[K], npan);
            mark(2);
            grid.sync();
            mark(3);
            if (bid == 0) store_diag(k0, kb);  // no block reads A_KK any more
        }
    } else {
        for (int K = 0; K < nt; ++K) {
            const int k0 = K * kTile, kb = min(kTile, m - k0);
            const int npan = pan_off[K + 1] - pan_off[K];
            if (bid == 0 || bid < npan) column(K, false);
            grid.sync();
            mark(3);
            if (bid == 0) store_diag(k0, kb);  // every block has read A_KK
            trailing(K, tr_off[K], tr_off[K + 1], npan);
            mark(2);
            grid.sync();
            mark(3);
        }
    }
    // the inverses of the diagonal tiles, a tile per block
    grid.sync();
    for (int K = bid; K < nt; K += nb) {
        const int k0 = K * kTile, kb = min(kTile, m - k0);
        __syncthreads();
        tile_load(tk, S, m, k0, kb, k0, kb, true);
        if (tid < kTile) rv[tid] = tid < kb ? rinv[k0 + tid] : T(1);
        __syncthreads();
        if (wid == 0) invert_diag_tile(tk, rv, DI + (size_t)K * 2 * kTile * kTile);
    }
    mark(4);
    if (timed)
        for (int k = 0; k < 5; ++k) phase[k] += tacc[k];
    if (bad) atomicOr(&sbad, 1);
    __syncthreads();
    if (tid == 0 && sbad) fail[0] = 1;
}

// Asynchronous global -> shared copies (cp.async, completed through commit groups).
__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"((unsigned)__cvta_generic_to_shared(dst)), "l"(src));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N));
}

// Triangular solves: the shared-memory ring of tile steps (kSolveRing slots).  A slot holds one
// step's diagonal-tile inverse (forward L^-T, backward L^-1; 32 x 32) and up to P panel tiles of
// the step's column (forward: transposed, from LT; backward: as is, from LN), all contiguous.
constexpr int kSolveRing = 3;
template <class T>
__host__ __device__ constexpr size_t solve_slot_elems(int P) {
    return (size_t)(1 + P) * kTile * kTile;
}

// Solve L L^T x = b in place (one CTA of 512 threads), tile by tile inside the envelope: the
// forward sweep then the backward sweep, 2 nt tile steps.  The data of step i + 2 (its diagonal
// tile's inverse and panel tiles, contiguous copies the factorization left) is copied into the
// shared-memory ring with 16-byte cp.async while step i runs: on GB300 an L2 round trip (~1.5k
// cycles) is longer than a tile step, and loading a step's data one step ahead left that latency
// on the serial chain (78 us of a 146 us solve on the 200-camera grid with its panel work removed).
// - Warp 0 applies the diagonal tile's inverse as a 32 x 32 product, lane per output.
// - Warps 1..15 take the column's panel tiles (rows(K)), a tile per warp.  Forward,
//   x_r -= L_r,K x_K: lane per row over the transposed tile (no cross-lane reduction: a warp
//   shuffle issues at one per SM clock on GB300).  Backward, x_K -= sum_r L_r,K^T x_r: lane per
//   column over the tile's rows; then over warps in order.  Tiles beyond the P a slot holds are
//   read from global memory.  Warp 0 copies nothing: it carries the serial chain.
// Every shared-memory read is a row of a block with lanes over its columns (conflict-free), every
// sum runs in four partial sums (index mod 4).  Bitwise repeatable.  kXs: x is kept in dynamic
// shared memory (padded with zeros to whole tiles) ahead of the ring.  The mixed form's refinement
// converts on the way: with b_in, x starts as b_in rounded to T (xg's contents are not read); with
// x_out, x_out = x_add + x in FP64 at the end (x also stored into xg).
template <class T, bool kXs>
__global__ void __launch_bounds__(512) k_chol_solve(const T* __restrict__ LT, const T* __restrict__ LN,
                                                    const T* __restrict__ DI, int m, const int32_t* __restrict__ pan_off,
                                                    const int32_t* __restrict__ pan_row, T* __restrict__ xg, int P,
                                                    const double* __restrict__ b_in, const T* __restrict__ x_add,
                                                    double* __restrict__ x_out) {
    constexpr int kW = 16;  // warps
    constexpr int kPer16 = 16 / sizeof(T);
    constexpr int kChunks = kTile * kTile / kPer16;  // 16-byte chunks per 32 x 32 block
    __shared__ T xk[kTile];
    __shared__ T red[kW][kTile + 1];
    extern __shared__ __align__(16) unsigned char dyn_raw[];
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const int nt = (m + kTile - 1) / kTile;
    if (nt == 0) return;
    T* const xs = reinterpret_cast<T*>(dyn_raw);
    T* const ring = xs + (kXs ? (size_t)nt * kTile : 0);
    const size_t slot_elems = solve_slot_elems<T>(P);
    T* x = kXs ? xs : xg;
    if constexpr (kXs) {
        for (int i = tid; i < nt * kTile; i += blockDim.x) x[i] = i < m ? (b_in ? (T)b_in[i] : xg[i]) : T(0);
    } else {
        if (b_in) {
            for (int i = tid; i < m; i += blockDim.x) x[i] = (T)b_in[i];
        }
    }
    auto xrow = [&](int r) -> T { return kXs ? x[r] : x[min(r, m - 1)]; };
    const int nsteps = 2 * nt;
    auto step_col = [&](int i) { return i < nt ? i : nsteps - 1 - i; };
    // copies step i's blocks into its ring slot (warps 1..15), one commit group per thread
    auto issue = [&](int i) {
        if (i < nsteps && wid > 0) {
            const bool fwd = i < nt;
            const int K = step_col(i);
            T* sl = ring + (size_t)(i % kSolveRing) * slot_elems;
            const int p0 = pan_off[K], n = min(pan_off[K + 1] - p0, P);
            const T* di = DI + ((size_t)2 * K + (fwd ? 0 : 1)) * kTile * kTile;
            const T* src = fwd ? LT : LN;
            for (int e = tid - kTile; e < (1 + n) * kChunks; e += blockDim.x - kTile) {
                const int b = e / kChunks, q = e % kChunks;
                const T* g = b == 0 ? di + q * kPer16 : src + (size_t)(p0 + b - 1) * kTile * kTile + q * kPer16;
                cp_async16(sl + (size_t)b * kTile * kTile + q * kPer16, g);
            }
        }
        cp_async_commit();
    };
    for (int i = 0; i < kSolveRing - 1; ++i) issue(i);
    for (int i = 0; i < nsteps; ++i) {
        cp_async_wait<kSolveRing - 2>();  // step i's group is complete
        __syncthreads();                   // ... for every thread; slot (i - 1) is free
        issue(i + kSolveRing - 1);
        const bool fwd = i < nt;
        const int K = step_col(i), k0 = K * kTile, kb = min(kTile, m - k0);
        const T* sl = ring + (size_t)(i % kSolveRing) * slot_elems;
        const T* tl = sl + kTile * kTile;
        const int p0 = pan_off[K], npan = pan_off[K + 1] - p0;
        if (!fwd && wid > 0) {  // backward: sum_r L_r,K^T x_r over the panel rows
            T a4[4] = {T(0), T(0), T(0), T(0)};  // four partial sums (row mod 4)
            for (int t = wid - 1; t < npan; t += kW - 1) {
                const int r0 = pan_row[p0 + t] * kTile;
                const T* ln = t < P ? tl + (size_t)t * kTile * kTile : LN + (size_t)(p0 + t) * kTile * kTile;
#pragma unroll
                for (int c = 0; c < kTile; ++c) a4[c & 3] += ln[c * kTile + lane] * xrow(r0 + c);
            }
            red[wid][lane] = (a4[0] + a4[1]) + (a4[2] + a4[3]);
        }
        if (!fwd) __syncthreads();
        if (wid == 0) {
            // x_K = L_KK^-1 b_K (forward; block L^-T) or L_KK^-T (y_K - sum) (backward; block L^-1):
            // v_lane = sum_j block[j][lane] u_j
            T u = lane < kb ? x[k0 + lane] : T(0);
            if (!fwd) {
                T s4[4] = {T(0), T(0), T(0), T(0)};
#pragma unroll
                for (int w = 1; w < kW; ++w) s4[w & 3] += red[w][lane];
                u -= (s4[0] + s4[1]) + (s4[2] + s4[3]);
                if (lane >= kb) u = T(0);
            }
            xk[lane] = u;
            __syncwarp();
            T v4[4] = {T(0), T(0), T(0), T(0)};
#pragma unroll
            for (int j = 0; j < kTile; ++j) v4[j & 3] += sl[j * kTile + lane] * xk[j];
            const T v = (v4[0] + v4[1]) + (v4[2] + v4[3]);
            __syncwarp();
            if (lane < kb) x[k0 + lane] = v;
            xk[lane] = lane < kb ? v : T(0);
        }
        if (fwd) {
            __syncthreads();
            if (wid > 0) {  // forward: x_r -= L_r,K x_K over the panel rows
                for (int t = wid - 1; t < npan; t += kW - 1) {
                    const int r = pan_row[p0 + t] * kTile + lane;
                    const T* lt = t < P ? tl + (size_t)t * kTile * kTile : LT + (size_t)(p0 + t) * kTile * kTile;
                    T s4[4] = {T(0), T(0), T(0), T(0)};
#pragma unroll
                    for (int c = 0; c < kTile; ++c) s4[c & 3] += lt[c * kTile + lane] * xk[c];
                    if (r < m) x[r] -= (s4[0] + s4[1]) + (s4[2] + s4[3]);
                }
            }
        }
    }
    cp_async_wait<0>();
    __syncthreads();
    if constexpr (kXs) {
        for (int i = tid; i < m; i += blockDim.x) xg[i] = x[i];
    }
    if (x_out)
        for (int i = tid; i < m; i += blockDim.x) x_out[i] = (double)x_add[i] + (double)x[i];
}

// Launches the triangular solves of a factored S: x in shared memory when it fits beside a ring
// of at least one panel tile per slot (NAVBA_SOLVE_GLOBAL_X=1 keeps it in global memory, the form
// for larger systems, to test it); each ring slot holds up to max_npan panel tiles, as many as
// the shared-memory budget allows.
template <class T>
cudaError_t chol_solve(const T* LT, const T* LN, const T* DI, int m, const int32_t* pan_off, const int32_t* pan_row,
                       T* x, int max_npan, cudaStream_t st, const double* b_in = nullptr, const T* x_add = nullptr,
                       double* x_out = nullptr) {
    const char* gx = getenv("NAVBA_SOLVE_GLOBAL_X");
    const bool global_x = gx && gx[0] == '1';
    const size_t xs_bytes = sizeof(T) * (size_t)std::max(1, (m + kTile - 1) / kTile * kTile);
    auto ring_bytes = [](int P) { return kSolveRing * solve_slot_elems<T>(P) * sizeof(T); };
    const bool use_xs = !global_x && xs_bytes + ring_bytes(1) <= kSolveSmem;
    const size_t budget = kSolveSmem - (use_xs ? xs_bytes : 0);
    int P = std::max(0, max_npan);
    while (P > 0 && ring_bytes(P) > budget) --P;
    const size_t smem = (use_xs ? xs_bytes : 0) + ring_bytes(P);
    cudaError_t e;
    if (use_xs) {
        e = cudaFuncSetAttribute(k_chol_solve<T, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        k_chol_solve<T, true><<<1, 512, smem, st>>>(LT, LN, DI, m, pan_off, pan_row, x, P, b_in, x_add, x_out);
    } else {
        e = cudaFuncSetAttribute(k_chol_solve<T, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        k_chol_solve<T, false><<<1, 512, smem, st>>>(LT, LN, DI, m, pan_off, pan_row, x, P, b_in, x_add, x_out);
    }
    return cudaGetLastError();
}


// r = b - S x in FP64 (warp per row of the mirrored S), rounded to FP32; x in FP32.
// Row i runs over the symmetric envelope only, tiles tfirst[i / 32] .. tlast[i / 32] (whole tiles,
// so each lane sums the same terms in the same order as over the whole row, less zeros).
__global__ void k_s_residual(const double* S, const float* x, const double* b, int m, const int32_t* tfirst,
                             const int32_t* tlast, float* r) {
    const CC c = grid_view();
    for (int i = c.gw; i < m; i += c.CW) {
        const double* Si = S + (size_t)i * m;
        const int lo = tfirst[i / kTile] * kTile, hi = min(m, (tlast[i / kTile] + 1) * kTile);
        double acc = 0.0;
        for (int j = lo + c.lane; j < hi; j += 32) acc += Si[j] * (double)x[j];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(kFullG, acc, o);
        if (c.lane == 0) r[i] = (float)(b[i] - acc);
    }
}

// Camera k: trial = exp(dx_a) * current when free; Real copy (and FP64 one into camd, when
// given); returns its term of the step scale dx^T (lambda dx + b).
template <class Real>
__device__ double update_camera(int k, const CamState* cur, CamState* trial, Real* camr_trial, const int32_t* cam_free,
                                const double* dc, const double* U, double lambda, double* camd) {
    double sc = 0.0;
    const int a = cam_free[k];
    if (a >= 0) {
        se3_left_update(dc + 6 * a, cur[k], trial[k]);
        for (int r = 0; r < 6; ++r) sc += dc[6 * a + r] * (lambda * dc[6 * a + r] + U[28LL * a + 21 + r]);
    } else {
        trial[k] = cur[k];
    }
    cam_real<Real>(trial[k], camr_trial + 12 * k);
    if (camd) cam_real<double>(trial[k], camd + 12 * k);
    return sc;
}

// Cameras, a thread per camera; scale part per block.
template <class Real>
__global__ void k_update_cams(const CamState* cur, CamState* trial, Real* camr_trial, const int32_t* cam_free, int nc,
                              const double* dc, const double* U, double lambda, double* part) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const double sc = k < nc ? update_camera<Real>(k, cur, trial, camr_trial, cam_free, dc, U, lambda, nullptr) : 0.0;
    block_partial<false>(sc, part);
}

// A damping trial's updates in one launch.  First a block per 32 cameras whose warp 0 alone works
// (a thread per camera, its warp's partial into part_c[g]): an FP64 instruction occupies its SM
// partition 64 cycles per warp whatever its active lanes, so the cameras' FP64 work (SE(3)
// exponential and products) is spread over as many SMs as there are warps of cameras; 200
// cameras in one 256-thread block (two warps per partition) took 28 us, and a launch of their own
// ~5 us more beside the points' launch.  Then npb blocks of points, as a launch of npb blocks of
// k_update_points would run them (its partials into part_p).  256 threads; at most 64 registers,
// so that four blocks fit per SM.
template <class Real>
__global__ void __launch_bounds__(256, 4)
    k_update_trial(WinArgs<Real> A, WinDesc D, double lambda, const double* dc, int cur, int ncb, int npb,
                   double* part_p, const CamState* cams_cur, CamState* cams_trial, Real* camr_trial,
                   const int32_t* cam_free, int nc, const double* U, double* part_c, double* camd) {
    if ((int)blockIdx.x >= ncb) {
        const int b = blockIdx.x - ncb;  // the point block
        CC c = grid_view();
        c.gt = b * blockDim.x + threadIdx.x;
        c.CT = npb * blockDim.x;
        c.gw = b * c.nw + c.wid;
        c.CW = npb * c.nw;
        block_partial<false>(update_points<Real>(A, c, D, lambda, dc, cur), part_p, b);
        return;
    }
    if (threadIdx.x >= 32) return;
    const int g = blockIdx.x, k = g * 32 + threadIdx.x;
    double sc =
        k < nc ? update_camera<Real>(k, cams_cur, cams_trial, camr_trial, cam_free, dc, U, lambda, camd) : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) sc += __shfl_down_sync(kFullG, sc, o);
    if (threadIdx.x == 0) part_c[g] = sc;
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


// ---- shared radial distortion (k1, k2) and the PCG solver ---------------------------------

// Block sums of N per-thread values; thread 0 writes out[N * blockIdx.x + k].
template <int N>
__device__ void block_partials(double (&v)[N], double* out) {
    __shared__ double red[32 * N];
#pragma unroll
    for (int k = 0; k < N; ++k)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_down_sync(kFullG, v[k], o);
    if ((threadIdx.x & 31) == 0)
#pragma unroll
        for (int k = 0; k < N; ++k) red[N * (threadIdx.x >> 5) + k] = v[k];
    __syncthreads();
    if (threadIdx.x == 0)
        for (int k = 0; k < N; ++k) {
            double r = 0.0;
            for (int i = 0; i < (int)(blockDim.x >> 5); ++i) r += red[N * i + k];
            out[N * blockIdx.x + k] = r;
        }
}

// Intrinsics rows of H: per free point Kp = sum w Jk^T Jp (2x3); block sums of H_kk (3 unique)
// and g_k (2) over every edge (the shared intrinsics are a free vertex of every edge).
template <class Real>
__global__ void k_lin_intr_points(WinArgs<Real> A, WinDesc D, const Real* camr, const double* X, Real* pt_kp,
                                  double* part) {
    const CC c = grid_view();
    const Real delta = (Real)A.lm.huber_delta;
    double acc[5] = {0, 0, 0, 0, 0};
    for (int p = c.gt; p < D.npt; p += c.CT) {
        const bool fp = A.pt_free[p] >= 0;
        const Real Xr[3] = {(Real)X[4LL * p], (Real)X[4LL * p + 1], (Real)X[4LL * p + 2]};
        Real kp[6] = {0, 0, 0, 0, 0, 0};
        for (int e = A.pt_eoff[p]; e < A.pt_eoff[p + 1]; ++e) {
            const Real* cr = camr + 12 * A.edge_cam[e];
            const Real z[2] = {(Real)A.edge_uv[2LL * e], (Real)A.edge_uv[2LL * e + 1]};
            EdgeLin<Real> L;
            edge_linearize_e<Real>(A, e, cr, Xr, z, delta, L);
            const Real w = L.w;
            const Real* jk = L.jk;  // rows: residual u, v; columns: k1, k2
            acc[0] += (double)(w * (jk[0] * jk[0] + jk[2] * jk[2]));
            acc[1] += (double)(w * (jk[0] * jk[1] + jk[2] * jk[3]));
            acc[2] += (double)(w * (jk[1] * jk[1] + jk[3] * jk[3]));
            acc[3] += (double)(-w * (jk[0] * L.e[0] + jk[2] * L.e[1]));
            acc[4] += (double)(-w * (jk[1] * L.e[0] + jk[3] * L.e[1]));
            if (fp)
#pragma unroll
                for (int r = 0; r < 2; ++r)
#pragma unroll
                    for (int q = 0; q < 3; ++q) kp[r * 3 + q] += w * (jk[r] * L.jp[q] + jk[2 + r] * L.jp[3 + q]);
        }
        if (fp) {
            const Real v[12] = {kp[0], kp[1], kp[2], kp[3], kp[4], kp[5], 0, 0, 0, 0, 0, 0};
            Rec<Real>::store12(pt_kp + 12LL * p, v);
        }
    }
    block_partials<5>(acc, part);
}

// Camera-intrinsics blocks: per work item sum w Jc^T Jk (6x2) -> hpart[item] (12 values).
template <class Real>
__global__ void k_lin_intr_cams(WinArgs<Real> A, const int4* items, int n_items, const int32_t* cam_list,
                                const int32_t* fcam, const Real* camr, const double* X, double* hpart) {
    const CC c = grid_view();
    const Real delta = (Real)A.lm.huber_delta;
    for (int it = c.gw; it < n_items; it += c.CW) {
        const int4 wi = items[it];
        const Real* cr = camr + 12 * fcam[wi.x];
        Real h[12];
#pragma unroll
        for (int k = 0; k < 12; ++k) h[k] = Real(0);
        for (int i = c.lane; i < wi.z; i += 32) {
            const int e = cam_list[wi.y + i];
            const int gp = A.edge_pt[e];
            const Real Xr[3] = {(Real)X[4LL * gp], (Real)X[4LL * gp + 1], (Real)X[4LL * gp + 2]};
            const Real z[2] = {(Real)A.edge_uv[2LL * e], (Real)A.edge_uv[2LL * e + 1]};
            EdgeLin<Real> L;
            edge_linearize_e<Real>(A, e, cr, Xr, z, delta, L);
#pragma unroll
            for (int r = 0; r < 6; ++r)
#pragma unroll
                for (int q = 0; q < 2; ++q) h[r * 2 + q] += L.w * (L.jc[r] * L.jk[q] + L.jc[6 + r] * L.jk[2 + q]);
        }
#pragma unroll
        for (int k = 0; k < 12; ++k)
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) h[k] += __shfl_xor_sync(kFullG, h[k], o);
        const Real hk = lane_value<12>(h, c.lane);
        if (c.lane < 12) hpart[12LL * it + c.lane] = (double)hk;
    }
}

// Per-camera sums of item partials (stride `stride`, first `nval` values) in item order.
__global__ void k_reduce_items(const double* part, int stride, int nval, const int32_t* item_off, int nfc, double* out,
                               int out_stride) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= nfc * nval) return;
    const int a = idx / nval, k = idx % nval;
    double s = 0.0;
    for (int it = item_off[a]; it < item_off[a + 1]; ++it) s += part[(long long)stride * it + k];
    out[(long long)out_stride * a + k] = s;
}

// Per free point: B = Kp L^T (2x3); block sums of B B^T (3 unique) and B t (2).
template <class Real>
__global__ void k_schur_intr_points(WinArgs<Real> A, WinDesc D, const Real* pt_kp, Real* pt_b, double* part) {
    const CC c = grid_view();
    double acc[5] = {0, 0, 0, 0, 0};
    for (int p = c.gt; p < D.npt; p += c.CT) {
        if (A.pt_free[p] < 0) continue;
        Real kp[12], lt[12];
        Rec<Real>::load12(pt_kp + 12LL * p, kp);
        Rec<Real>::load12(A.pt_lt + 12LL * p, lt);
        // L packed lower: l00 lt[0], l10 lt[1], l11 lt[2], l20 lt[3], l21 lt[4], l22 lt[5]; B = Kp L^T
        Real b[6];
#pragma unroll
        for (int r = 0; r < 2; ++r) {
            const Real k0 = kp[r * 3], k1 = kp[r * 3 + 1], k2 = kp[r * 3 + 2];
            b[r * 3 + 0] = k0 * lt[0];
            b[r * 3 + 1] = k0 * lt[1] + k1 * lt[2];
            b[r * 3 + 2] = k0 * lt[3] + k1 * lt[4] + k2 * lt[5];
        }
        const Real v[12] = {b[0], b[1], b[2], b[3], b[4], b[5], 0, 0, 0, 0, 0, 0};
        Rec<Real>::store12(pt_b + 12LL * p, v);
        acc[0] += (double)(b[0] * b[0] + b[1] * b[1] + b[2] * b[2]);
        acc[1] += (double)(b[0] * b[3] + b[1] * b[4] + b[2] * b[5]);
        acc[2] += (double)(b[3] * b[3] + b[4] * b[4] + b[5] * b[5]);
        acc[3] += (double)(b[0] * lt[6] + b[1] * lt[7] + b[2] * lt[8]);
        acc[4] += (double)(b[3] * lt[6] + b[4] * lt[7] + b[5] * lt[8]);
    }
    block_partials<5>(acc, part);
}

// Preconditioner and right-hand side, per work item over the camera lists: sum A A^T (21) and
// sum A t (6) -> part[28 * item].
template <class Real>
__global__ void k_pcg_diag_items(WinArgs<Real> A, const int4* items, int n_items, const int32_t* cam_list, double* part) {
    const CC c = grid_view();
    for (int it = c.gw; it < n_items; it += c.CW) {
        const int4 wi = items[it];
        Real u[27];
#pragma unroll
        for (int k = 0; k < 27; ++k) u[k] = Real(0);
        for (int i = c.lane; i < wi.z; i += 32) {
            const int e = cam_list[wi.y + i];
            const int gp = A.edge_pt[e];
            if (A.pt_free[gp] < 0) continue;
            Real a[18], lt[12];
            Rec<Real>::load18(A.edge_a + (long long)Rec<Real>::kEdge * e, a);
            Rec<Real>::load12(A.pt_lt + 12LL * gp, lt);
#pragma unroll
            for (int r = 0; r < 6; ++r) {
#pragma unroll
                for (int q = 0; q <= r; ++q) u[tri(r, q)] += a[r * 3] * a[q * 3] + a[r * 3 + 1] * a[q * 3 + 1] + a[r * 3 + 2] * a[q * 3 + 2];
                u[21 + r] += a[r * 3] * lt[6] + a[r * 3 + 1] * lt[7] + a[r * 3 + 2] * lt[8];
            }
        }
#pragma unroll
        for (int k = 0; k < 27; ++k)
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) u[k] += __shfl_xor_sync(kFullG, u[k], o);
        const Real uk = lane_value<27>(u, c.lane);
        if (c.lane < 27) part[28LL * it + c.lane] = (double)uk;
    }
}

// FP64 Cholesky of a packed 6x6 block in place (lower L) and 1/L_jj; false (with the pivot
// replaced by 1) if the block is not positive definite.
__device__ bool chol6_packed(double (&P)[21], double (&rinv)[6]) {
    bool good = true;
    for (int j = 0; j < 6; ++j) {
        double d = P[tri(j, j)];
        for (int k = 0; k < j; ++k) d -= P[tri(j, k)] * P[tri(j, k)];
        if (!(d > 0.0) || !isfinite(d)) {
            good = false;
            d = 1.0;
        }
        const double r = rsqrt(d);
        P[tri(j, j)] = d * r;
        rinv[j] = r;
        for (int i = j + 1; i < 6; ++i) {
            double v = P[tri(i, j)];
            for (int k = 0; k < j; ++k) v -= P[tri(i, k)] * P[tri(j, k)];
            P[tri(i, j)] = v * r;
        }
    }
    return good;
}

// Per free camera: P_a = U_a + lambda I - sum A A^T, FP64 Cholesky (packed lower L, with 1/L_jj in
// the diagonal slots of pinv); b'_a = g_a - sum A t.  pc[28 a]: 21 L entries + 6 inverse diagonal.
__global__ void k_pcg_precond(const double* U, const double* aat, int nfc, double lambda, double* pc, double* b,
                              int32_t* ok) {
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= nfc) return;
    double P[21];
    for (int k = 0; k < 21; ++k) P[k] = U[28LL * a + k] - aat[28LL * a + k];
    for (int r = 0; r < 6; ++r) P[tri(r, r)] += lambda;
    double rinv[6];
    const bool good = chol6_packed(P, rinv);
    for (int k = 0; k < 21; ++k) pc[28LL * a + k] = P[k];
    for (int k = 0; k < 6; ++k) pc[28LL * a + 21 + k] = rinv[k];
    for (int k = 0; k < 6; ++k) b[6 * a + k] = U[28LL * a + 21 + k] - aat[28LL * a + 21 + k];
    if (!good) ok[0] = 0;
}

// The same block-Jacobi factor from the diagonal slots of the explicit S (lambda included).
// z = P_a^-1 r for camera a (6x6 Cholesky factors with inverse diagonal).
__device__ __forceinline__ void precond_cam(const double* pc, int a, const double* r, double* z) {
    const double* L = pc + 28LL * a;
    const double* ri = L + 21;
    double v[6];
    for (int i = 0; i < 6; ++i) {
        double s = r[i];
        for (int k = 0; k < i; ++k) s -= L[tri(i, k)] * v[k];
        v[i] = s * ri[i];
    }
    for (int i = 5; i >= 0; --i) {
        double s = v[i];
        for (int k = i + 1; k < 6; ++k) s -= L[tri(k, i)] * v[k];
        v[i] = s * ri[i];
    }
    for (int i = 0; i < 6; ++i) z[i] = v[i];
}

template <class Real>
__global__ void k_pcg_precond_blocks(const Real* Sb, const int32_t* dslot, int nfc, double* pc, double* pcinv,
                                     int32_t* ok) {
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= nfc) return;
    const Real* d = Sb + 36LL * dslot[a];
    double P[21];
    for (int r = 0; r < 6; ++r)
        for (int q = 0; q <= r; ++q) P[tri(r, q)] = (double)d[6 * r + q];
    double rinv[6];
    const bool good = chol6_packed(P, rinv);
    for (int k = 0; k < 21; ++k) pc[28LL * a + k] = P[k];
    for (int k = 0; k < 6; ++k) pc[28LL * a + 21 + k] = rinv[k];
    // the block's inverse (row-major 6 x 6), column by column through the factors
    for (int j = 0; j < 6; ++j) {
        double e[6] = {0, 0, 0, 0, 0, 0}, z[6];
        e[j] = 1.0;
        precond_cam(pc, a, e, z);
        for (int i = 0; i < 6; ++i) pcinv[36LL * a + 6 * i + j] = z[i];
    }
    if (!good) ok[0] = 0;
}

// Camera-k coupling of the reduced system, per work item over the camera lists: sum A_e B_p
// (6 x 2, entry r * 2 + j) -> part[12 * item]; S_ak = H_ck,a - the camera's sum.
template <class Real>
__global__ void k_pcg_xak_items(WinArgs<Real> A, const int4* items, int n_items, const int32_t* cam_list,
                                const Real* pt_b, double* part) {
    const CC c = grid_view();
    for (int it = c.gw; it < n_items; it += c.CW) {
        const int4 wi = items[it];
        Real u[12];
#pragma unroll
        for (int k = 0; k < 12; ++k) u[k] = Real(0);
        for (int i = c.lane; i < wi.z; i += 32) {
            const int e = cam_list[wi.y + i];
            const int gp = A.edge_pt[e];
            if (A.pt_free[gp] < 0) continue;
            Real a[18], bp[12];
            Rec<Real>::load18(A.edge_a + (long long)Rec<Real>::kEdge * e, a);
            Rec<Real>::load12(pt_b + 12LL * gp, bp);
#pragma unroll
            for (int r = 0; r < 6; ++r)
#pragma unroll
                for (int j = 0; j < 2; ++j)
                    u[2 * r + j] += a[3 * r] * bp[3 * j] + a[3 * r + 1] * bp[3 * j + 1] + a[3 * r + 2] * bp[3 * j + 2];
        }
#pragma unroll
        for (int k = 0; k < 12; ++k)
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) u[k] += __shfl_xor_sync(kFullG, u[k], o);
        const Real uk = lane_value<12>(u, c.lane);
        if (c.lane < 12) part[12LL * it + c.lane] = (double)uk;
    }
}

// Structure-of-arrays copies of A_e for the PCG products (18 arrays of Real each): point-major in
// edge order (apm[k * ne + e]) and camera-major in camera-list order (acm[k * ncl + s]), packed
// once per damping trial from the per-edge records and read by every PCG iteration with
// contiguous (coalesced) accesses.  Entries of edges without a free camera or a free point are
// not written and never read.
template <class Real>
__global__ void k_pcg_pack(WinArgs<Real> A, int ne, const int32_t* cam_list, int ncl, Real* apm, Real* acm) {
    const int stride = gridDim.x * blockDim.x;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < ne; e += stride) {
        if (A.edge_fc[e] < 0 || A.pt_free[A.edge_pt[e]] < 0) continue;
        Real a[18];
        Rec<Real>::load18(A.edge_a + (long long)Rec<Real>::kEdge * e, a);
#pragma unroll
        for (int k = 0; k < 18; ++k) apm[(long long)k * ne + e] = a[k];
    }
    for (int sl = blockIdx.x * blockDim.x + threadIdx.x; sl < ncl; sl += stride) {
        const int e = cam_list[sl];
        if (A.pt_free[A.edge_pt[e]] < 0) continue;
        Real a[18];
        Rec<Real>::load18(A.edge_a + (long long)Rec<Real>::kEdge * e, a);
#pragma unroll
        for (int k = 0; k < 18; ++k) acm[(long long)k * ncl + sl] = a[k];
    }
}

// PCG vectors x r z p q of length mt and scalars.
struct PcgVec {
    double *x, *r, *z, *p, *q;
    double* sc;  // [0] rz, [1] r.r, [2] b.b
    float* pf;   // FP32 copy of the camera part of p (mixed form), or null
    int npf;     // its length (6 * free cameras)
};

// ---- PCG as one cooperative persistent kernel ------------------------------------------------
//
// One launch per damped system: every phase of every CG iteration runs grid-wide with grid
// synchronizations in between (no host round trip, no per-iteration launches).  Reductions go
// through per-block partials that every block sums in the same fixed order, so every block holds
// the same scalars and the iteration is bitwise repeatable.  The convergence test (r.r <= tol^2
// b.b) is made every 4 iterations, as in the oracle.

template <class Real>
struct PcgArgs {
    WinArgs<Real> A;
    int np, ne, ncl, nfc, nk, mt;
    const Real* apm;
    const Real* acm;
    const int32_t* cm_pt;
    const int4* items;
    int n_items;
    const int32_t* item_off;
    const Real* pt_b;
    Real* pt_t2;
    double* camp;           // [n_items][8]
    const double* U;        // [nfc][28]
    const double* Hck;      // [nfc][12]
    const double* kk;       // [0..2] H_kk (lambda-free), [3..5] 2x2 Cholesky of the k block
    const double* pc;       // [nfc][28] block-Jacobi factors
    const double* b;        // right-hand side [mt]
    double lambda;
    PcgVec v;
    double* part;           // [7][gridDim.x] partials
    int max_it;
    double tol2;
    int32_t* iters;         // out: iterations run
    unsigned long long* phase;  // optional: SM cycles of the five phases (block 0 after each sync), or null
};

// Sum of n per-block partials (stride `stride`) in a fixed order; every thread gets the result.
__device__ double grid_partials_sum(const double* part, int n, int stride) {
    __shared__ double red[32];
    double v = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) v += part[(long long)i * stride];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(kFullG, v, o);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    double r = 0.0;
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) r += red[i];
    __syncthreads();
    return r;
}

// Reductions of the explicit PCG whose FP64 adds run in warp 0 alone (the FP64 pipe is shared by
// the SM and charged per warp instruction; the other warps only stage or read values).  Orders are
// fixed: every block gets the same bits.
// Block sum of N doubles per thread (blockDim.x <= 256); warp 0 writes out[N * blockIdx.x + k].
template <int N>
__device__ void block_sum_w0(const double (&v)[N], double* out) {
    __shared__ double stage[N][256];
#pragma unroll
    for (int k = 0; k < N; ++k) stage[k][threadIdx.x] = v[k];
    __syncthreads();
    if (threadIdx.x < 32) {
#pragma unroll
        for (int k = 0; k < N; ++k) {
            double s = 0.0;
            for (int i = threadIdx.x; i < (int)blockDim.x; i += 32) s += stage[k][i];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(kFullG, s, o);
            if (threadIdx.x == 0) out[N * blockIdx.x + k] = s;
        }
    }
    __syncthreads();
}

// The N sums of per-block partials laid out [block][N], returned to every thread.
template <int N>
__device__ void grid_sum_w0(const double* part, int n, double (&out)[N]) {
    __shared__ double res[N];
    if (threadIdx.x < 32) {
#pragma unroll
        for (int k = 0; k < N; ++k) {
            double s = 0.0;
#pragma unroll 4
            for (int i = threadIdx.x; i < n; i += 32) s += part[(long long)i * N + k];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(kFullG, s, o);
            if (threadIdx.x == 0) res[k] = s;
        }
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < N; ++k) out[k] = res[k];
    __syncthreads();
}

// z = P_k^-1 r for the 2x2 intrinsics block (lower Cholesky l00 l10 l11 in pk).
__device__ __forceinline__ void precond_k(const double* pk, const double* r, double* z) {
    const double y0 = r[0] / pk[0];
    const double y1 = (r[1] - pk[1] * y0) / pk[2];
    const double x1 = y1 / pk[2];
    const double x0 = (y0 - pk[1] * x1) / pk[0];
    z[0] = x0;
    z[1] = x1;
}

template <class Real>
__global__ void __launch_bounds__(256) k_pcg_solve(PcgArgs<Real> P) {
    cg::grid_group grid = cg::this_grid();
    const int tid = blockIdx.x * blockDim.x + threadIdx.x, nth = gridDim.x * blockDim.x;
    const int nb = gridDim.x;
    const int lane = threadIdx.x & 31;
    const int gw = tid >> 5, nwarp = nth >> 5;
    const int kb = 6 * P.nfc;
    PcgVec& v = P.v;
    double* pk_part = P.part;               // phase 1: B t2 (2 per block)
    double* hk_part = P.part + 2LL * nb;    // phase 2: Hck^T p (2 per block)
    double* pq_part = P.part + 4LL * nb;    // phase 3: p.q
    double* rz_part = P.part + 5LL * nb;    // phase 4: r.z, r.r (2 per block)
    const double* pkc = P.kk + 3;
    long long tmark = clock64();
    auto mark = [&](int k) {  // phase timer: block 0's view, taken after the grid synchronization
        if (!P.phase || blockIdx.x != 0 || threadIdx.x != 0) return;
        const long long now = clock64();
        P.phase[k] += (unsigned long long)(now - tmark);
        tmark = now;
    };
    // init: x = 0, r = b, z = M^-1 r, p = z
    double rz = 0.0, rr = 0.0;
    for (int a = tid; a < P.nfc; a += nth) {
        double* r = v.r + 6 * a;
        for (int i = 0; i < 6; ++i) {
            v.x[6 * a + i] = 0.0;
            r[i] = P.b[6 * a + i];
        }
        precond_cam(P.pc, a, r, v.z + 6 * a);
        for (int i = 0; i < 6; ++i) {
            const double z = v.z[6 * a + i];
            v.p[6 * a + i] = z;
            if (v.pf) v.pf[6 * a + i] = (float)z;
            rz += r[i] * z;
            rr += r[i] * r[i];
        }
    }
    if (P.nk && tid == 0) {
        for (int i = 0; i < 2; ++i) {
            v.x[kb + i] = 0.0;
            v.r[kb + i] = P.b[kb + i];
        }
        precond_k(pkc, v.r + kb, v.z + kb);
        for (int i = 0; i < 2; ++i) {
            v.p[kb + i] = v.z[kb + i];
            rz += v.r[kb + i] * v.z[kb + i];
            rr += v.r[kb + i] * v.r[kb + i];
        }
    }
    {
        double two[2] = {rz, rr};
        block_partials<2>(two, rz_part);
    }
    grid.sync();
    rz = grid_partials_sum(rz_part, nb, 2);
    rr = grid_partials_sum(rz_part + 1, nb, 2);
    const double bb = rr;
    const Real* xr = reinterpret_cast<const Real*>(sizeof(Real) == 4 ? (const void*)v.pf : (const void*)v.p);
    int pit = 0;
    for (; pit < P.max_it; ++pit) {
        if (pit % 4 == 0 && !(rr > P.tol2 * bb)) break;
        // phase 1: t2_p = sum A_e^T p_c + B_p^T p_k (8 lanes per point, warp-uniform loop)
        {
            constexpr int G = 8, GPW = 32 / G;
            const int gl = lane % G, gi = lane / G;
            // B^T t2 partials in Real with Kahan compensation, widened once at the end: only the
            // group leaders hold them, and FP64 operations are charged per warp instruction
            Real ks[2] = {Real(0), Real(0)}, kc[2] = {Real(0), Real(0)};
            auto kahan = [&](int i, Real v) {
                const Real y = v - kc[i];
                const Real t = ks[i] + y;
                kc[i] = (t - ks[i]) - y;
                ks[i] = t;
            };
            const Real k1 = P.nk ? (Real)v.p[kb] : Real(0), k2 = P.nk ? (Real)v.p[kb + 1] : Real(0);
            for (int p0 = gw * GPW; p0 < P.np; p0 += nwarp * GPW) {
                const int p = p0 + gi;
                const bool valid = p < P.np && P.A.pt_free[p] >= 0;
                Real t0 = 0, t1 = 0, t2 = 0;
                if (valid) {
                    const int e1 = P.A.pt_eoff[p + 1];
                    for (int e = P.A.pt_eoff[p] + gl; e < e1; e += G) {
                        const int a = P.A.edge_fc[e];
                        if (a < 0) continue;
                        const Real* xa = xr + 6 * a;
#pragma unroll
                        for (int r = 0; r < 6; ++r) {
                            const Real xv = xa[r];
                            t0 += P.apm[(long long)(r * 3) * P.ne + e] * xv;
                            t1 += P.apm[(long long)(r * 3 + 1) * P.ne + e] * xv;
                            t2 += P.apm[(long long)(r * 3 + 2) * P.ne + e] * xv;
                        }
                    }
                }
#pragma unroll
                for (int o = G / 2; o > 0; o >>= 1) {
                    t0 += __shfl_xor_sync(kFullG, t0, o);
                    t1 += __shfl_xor_sync(kFullG, t1, o);
                    t2 += __shfl_xor_sync(kFullG, t2, o);
                }
                if (valid && gl == 0) {
                    if (P.nk) {
                        Real bp[12];
                        Rec<Real>::load12(P.pt_b + 12LL * p, bp);
                        t0 += bp[0] * k1 + bp[3] * k2;
                        t1 += bp[1] * k1 + bp[4] * k2;
                        t2 += bp[2] * k1 + bp[5] * k2;
                        kahan(0, bp[0] * t0 + bp[1] * t1 + bp[2] * t2);
                        kahan(1, bp[3] * t0 + bp[4] * t1 + bp[5] * t2);
                    }
                    P.pt_t2[4LL * p] = t0;
                    P.pt_t2[4LL * p + 1] = t1;
                    P.pt_t2[4LL * p + 2] = t2;
                }
            }
            double acc[2] = {(double)ks[0] - (double)kc[0], (double)ks[1] - (double)kc[1]};
            block_partials<2>(acc, pk_part);
        }
        grid.sync();
        mark(0);
        // phase 2: per camera item sum A_s t2 (warp per item); Hck_a^T p_a partials
        for (int it = gw; it < P.n_items; it += nwarp) {
            const int4 wi = P.items[it];
            Real y[6] = {0, 0, 0, 0, 0, 0};
            for (int i = lane; i < wi.z; i += 32) {
                const int sl = wi.y + i;
                const int gp = P.cm_pt[sl];
                if (gp < 0) continue;
                const Real t0 = P.pt_t2[4LL * gp], t1 = P.pt_t2[4LL * gp + 1], t2 = P.pt_t2[4LL * gp + 2];
#pragma unroll
                for (int r = 0; r < 6; ++r)
                    y[r] += P.acm[(long long)(r * 3) * P.ncl + sl] * t0 + P.acm[(long long)(r * 3 + 1) * P.ncl + sl] * t1 +
                            P.acm[(long long)(r * 3 + 2) * P.ncl + sl] * t2;
            }
#pragma unroll
            for (int k = 0; k < 6; ++k)
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) y[k] += __shfl_xor_sync(kFullG, y[k], o);
            const Real yk = lane_value<6>(y, lane);  // one FP64 conversion per warp, not per value
            if (lane < 6) P.camp[8LL * it + lane] = (double)yk;
        }
        {
            double hk[2] = {0, 0};
            if (P.nk)
                for (int a = tid; a < P.nfc; a += nth)
                    for (int r = 0; r < 6; ++r) {
                        hk[0] += P.Hck[12LL * a + r * 2] * v.p[6 * a + r];
                        hk[1] += P.Hck[12LL * a + r * 2 + 1] * v.p[6 * a + r];
                    }
            block_partials<2>(hk, hk_part);
        }
        grid.sync();
        mark(1);
        // phase 3: q = S p per camera (and the k block), p.q partials
        {
            double pq = 0.0;
            const double pk0 = P.nk ? v.p[kb] : 0.0, pk1 = P.nk ? v.p[kb + 1] : 0.0;
            for (int a = tid; a < P.nfc; a += nth) {
                const double* Ua = P.U + 28LL * a;
                double pa[6];
                for (int r = 0; r < 6; ++r) pa[r] = v.p[6 * a + r];
                for (int r = 0; r < 6; ++r) {
                    double s = P.lambda * pa[r];
                    for (int q = 0; q < 6; ++q) s += Ua[r >= q ? tri(r, q) : tri(q, r)] * pa[q];
                    for (int it = P.item_off[a]; it < P.item_off[a + 1]; ++it) s -= P.camp[8LL * it + r];
                    if (P.nk) s += P.Hck[12LL * a + r * 2] * pk0 + P.Hck[12LL * a + r * 2 + 1] * pk1;
                    v.q[6 * a + r] = s;
                    pq += pa[r] * s;
                }
            }
            if (P.nk) {
                // q_k = (H_kk + lambda) p_k + sum_a Hck_a^T p_a - sum_p B t2 (block 0 writes it)
                const double h0 = grid_partials_sum(hk_part, nb, 2), h1 = grid_partials_sum(hk_part + 1, nb, 2);
                const double b0 = grid_partials_sum(pk_part, nb, 2), b1 = grid_partials_sum(pk_part + 1, nb, 2);
                if (blockIdx.x == 0 && threadIdx.x == 0) {
                    const double q0 = (P.kk[0] + P.lambda) * pk0 + P.kk[1] * pk1 + h0 - b0;
                    const double q1 = P.kk[1] * pk0 + (P.kk[2] + P.lambda) * pk1 + h1 - b1;
                    v.q[kb] = q0;
                    v.q[kb + 1] = q1;
                    pq += pk0 * q0 + pk1 * q1;
                }
            }
            block_partial<false>(pq, pq_part);
        }
        grid.sync();
        mark(2);
        // phase 4: x += alpha p, r -= alpha q, z = M^-1 r, r.z and r.r partials
        {
            const double pq = grid_partials_sum(pq_part, nb, 1);
            const double alpha = pq != 0.0 ? rz / pq : 0.0;
            double rzn = 0.0, rrn = 0.0;
            for (int a = tid; a < P.nfc; a += nth) {
                double* r = v.r + 6 * a;
                for (int i = 0; i < 6; ++i) {
                    v.x[6 * a + i] += alpha * v.p[6 * a + i];
                    r[i] -= alpha * v.q[6 * a + i];
                }
                precond_cam(P.pc, a, r, v.z + 6 * a);
                for (int i = 0; i < 6; ++i) {
                    rzn += r[i] * v.z[6 * a + i];
                    rrn += r[i] * r[i];
                }
            }
            if (P.nk && tid == 0) {
                for (int i = 0; i < 2; ++i) {
                    v.x[kb + i] += alpha * v.p[kb + i];
                    v.r[kb + i] -= alpha * v.q[kb + i];
                }
                precond_k(pkc, v.r + kb, v.z + kb);
                for (int i = 0; i < 2; ++i) {
                    rzn += v.r[kb + i] * v.z[kb + i];
                    rrn += v.r[kb + i] * v.r[kb + i];
                }
            }
            double two[2] = {rzn, rrn};
            block_partials<2>(two, rz_part);
        }
        grid.sync();
        mark(3);
        // phase 5: p = z + beta p
        {
            const double rzn = grid_partials_sum(rz_part, nb, 2);
            rr = grid_partials_sum(rz_part + 1, nb, 2);
            const double beta = rz != 0.0 ? rzn / rz : 0.0;
            for (int i = tid; i < P.mt; i += nth) {
                const double pn = v.z[i] + beta * v.p[i];
                v.p[i] = pn;
                if (v.pf && i < kb) v.pf[i] = (float)pn;
            }
            rz = rzn;
        }
        grid.sync();
        mark(4);
    }
    if (tid == 0) P.iters[0] = pit;
}

// t_p -= B_p^T dk before the point back-substitution (the distortion part of the step).
// ---- PCG over the explicit reduced system --------------------------------------------------
//
// S in block rows of both triangles (36 Real per slot, row-major, lambda in the diagonal slots),
// S_ak = H_ck - sum A B per camera and S_kk (2 x 2) when the shared distortion is free.  One CG
// iteration is two grid-wide phases:
//   1. warp per camera row a: p_b = z_b + beta p_b (old) for every column camera b, computed by
//      each reader from z and the previous direction (the row's owner stores its own p_a in the
//      other buffer), q_a = sum_b S_ab p_b + S_ak p_k; partials of p.q and S_ka p
//   2. thread per camera: q_k, alpha = r.z / p.q, x += alpha p, r -= alpha q, z = M^-1 r;
//      partials of r.z and r.r
// so the direction update needs no grid synchronization of its own.  The block rows are a few
// MB (one camera's row: its co-observing cameras), read from L2 by every iteration; the
// per-observation records are read once per damping trial, when S is formed.  Sums run in the
// same fixed order in every block and every run.

template <class Real>
struct PcgXArgs {
    const Real* Sb;         // block rows, 36 per slot
    const int32_t* rs_off;  // first slot of each camera row (nfc + 1)
    const int32_t* rs_col;  // column camera of each slot
    const double* Hck;      // H_ck per camera (12, entry r * 2 + j), when nk
    const double* Xak;      // sum A B per camera (12), when nk
    const double* pcinv;    // block-Jacobi blocks' inverses (36 per camera, row-major)
    const double* kk;       // [3..5]: factor of the k block's preconditioner
    double skk[3];          // S_kk (00, 01, 11), lambda included
    const double* b;        // right-hand side (6 nfc + nk)
    double *x, *r, *z, *q;  // CG vectors
    double* p[2];           // directions, alternating
    Real* zr;               // z of the cameras in Real, 8 per camera (read by the products)
    Real* pr[2];            // the directions of the cameras in Real, 8 per camera
    double* part;           // per-block partials (5 per block)
    int nfc, nk, max_it;
    double tol2;
    int32_t* iters;
    unsigned long long* phase;  // optional: SM cycles per phase (block 0), or null
};

__device__ __forceinline__ void load36(const float* s, float (&v)[36]) {
    const float4* s4 = reinterpret_cast<const float4*>(s);
#pragma unroll
    for (int k = 0; k < 9; ++k) {
        const float4 t = s4[k];
        v[4 * k] = t.x;
        v[4 * k + 1] = t.y;
        v[4 * k + 2] = t.z;
        v[4 * k + 3] = t.w;
    }
}

__device__ __forceinline__ void load36(const double* s, double (&v)[36]) {
    const double2* s2 = reinterpret_cast<const double2*>(s);
#pragma unroll
    for (int k = 0; k < 18; ++k) {
        const double2 t = s2[k];
        v[2 * k] = t.x;
        v[2 * k + 1] = t.y;
    }
}

// The first 6 of a camera's 8 Real entries (32- or 64-byte aligned).
__device__ __forceinline__ void load6(const float* s, float (&v)[6]) {
    const float4 a = *reinterpret_cast<const float4*>(s);
    const float2 b = *reinterpret_cast<const float2*>(s + 4);
    v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w; v[4] = b.x; v[5] = b.y;
}

__device__ __forceinline__ void load6(const double* s, double (&v)[6]) {
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const double2 t = reinterpret_cast<const double2*>(s)[k];
        v[2 * k] = t.x;
        v[2 * k + 1] = t.y;
    }
}

template <class Real>
__global__ void __launch_bounds__(256, 2) k_pcg_explicit(PcgXArgs<Real> P) {
    cg::grid_group grid = cg::this_grid();
    const int tid = blockIdx.x * blockDim.x + threadIdx.x, nth = gridDim.x * blockDim.x;
    const int nb = gridDim.x;
    const int lane = threadIdx.x & 31;
    const int gw = tid >> 5, nwarp = nth >> 5;
    const int kb = 6 * P.nfc;
    double* mv_part = P.part;             // phase 1: p.q over the cameras, S_ka p (3 per block)
    double* rz_part = P.part + 3LL * nb;  // phase 2: r.z, r.r (2 per block)
    long long tmark = clock64();
    auto mark = [&](int k) {  // phase timer: block 0's view
        if (!P.phase || blockIdx.x != 0 || threadIdx.x != 0) return;
        const long long now = clock64();
        P.phase[k] += (unsigned long long)(now - tmark);
        tmark = now;
    };
    // per-camera work in chunks of 5 cameras per warp, lane per component (lanes 6g..6g+5: camera
    // 5c + g; lanes 30, 31 idle), spread over the blocks first.  An FP64 instruction costs its SM
    // partition 64 cycles per warp whatever its active lanes, so a camera's six components go across
    // lanes (an FP64 instruction per warp for all of them) rather than down one lane's registers (six
    // or more); the block-Jacobi inverse is applied as a row per lane against the group's residual.
    // Each lane's values are read into registers before anything is stored (the vectors may alias
    // as far as the compiler knows).
    const int nchunk = (P.nfc + 4) / 5, wib = threadIdx.x >> 5, nwb = blockDim.x >> 5;
    const int grp = lane / 6, comp = lane - 6 * grp, glead = 6 * min(grp, 4);
    // z_comp = (M_a^-1 r)_comp from the group's six residual components (all lanes shuffle)
    auto apply_inv = [&](int a, bool act, double rv) {
        const double* mi = P.pcinv + 36LL * (act ? a : 0) + 6 * (act ? comp : 0);
        double z = 0.0;
#pragma unroll
        for (int k = 0; k < 6; ++k) {
            const double rk = __shfl_sync(kFullG, rv, glead + k);
            z += mi[k] * rk;
        }
        return z;
    };
    // the k block's scalar work: thread 0 of the first block without a camera chunk
    const bool kthread = P.nk && threadIdx.x == 0 && blockIdx.x == min(nchunk, nb - 1);
    // k preconditioner: lower Cholesky l00 l10 l11 with the reciprocals of the diagonal
    const double l10 = P.kk[4], il00 = P.nk ? 1.0 / P.kk[3] : 0.0, il11 = P.nk ? 1.0 / P.kk[5] : 0.0;
    auto precond_k2 = [&](double r0, double r1, double& z0, double& z1) {
        const double y0 = r0 * il00;
        const double y1 = (r1 - l10 * y0) * il11;
        z1 = y1 * il11;
        z0 = (y0 - l10 * z1) * il00;
    };
    // Scalars of the iteration, reduced by warp 0 of every block (fixed order: the same bits in
    // every block) and broadcast through shared memory.
    __shared__ double sc[5];
    // init: x = 0, r = b, z = M^-1 r, previous direction 0 (the first direction is z)
    {
        double rz = 0.0, rr = 0.0;
        for (int c = blockIdx.x + nb * wib; c < nchunk; c += nb * nwb) {
            const int a = 5 * c + grp;
            const bool act = grp < 5 && a < P.nfc;
            const int i = 6 * a + comp;
            const double rv = act ? P.b[i] : 0.0;
            const double zv = apply_inv(a, act, rv);
            if (act) {
                P.x[i] = 0.0;
                P.p[0][i] = 0.0;
                P.r[i] = rv;
                P.z[i] = zv;
                P.zr[8 * a + comp] = (Real)zv;
                P.pr[0][8 * a + comp] = Real(0);
                rz += rv * zv;
                rr += rv * rv;
            }
        }
        if (kthread) {
            const double r0 = P.b[kb], r1 = P.b[kb + 1];
            double z0, z1;
            precond_k2(r0, r1, z0, z1);
            P.x[kb] = P.x[kb + 1] = 0.0;
            P.p[0][kb] = P.p[0][kb + 1] = 0.0;
            P.r[kb] = r0;
            P.r[kb + 1] = r1;
            P.z[kb] = z0;
            P.z[kb + 1] = z1;
            rz += r0 * z0 + r1 * z1;
            rr += r0 * r0 + r1 * r1;
        }
        double two[2] = {rz, rr};
        block_sum_w0<2>(two, rz_part);
    }
    grid.sync();
    if (threadIdx.x < 32) {
        double zk0 = 0.0, zk1 = 0.0;
        if (P.nk && lane == 0) {
            zk0 = P.z[kb];
            zk1 = P.z[kb + 1];
        }
        double s2[2] = {0.0, 0.0};
        for (int i = lane; i < nb; i += 32) {
            s2[0] += rz_part[2 * i];
            s2[1] += rz_part[2 * i + 1];
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            s2[0] += __shfl_down_sync(kFullG, s2[0], o);
            s2[1] += __shfl_down_sync(kFullG, s2[1], o);
        }
        if (lane == 0) {
            sc[0] = 0.0;    // beta
            sc[1] = s2[0];  // r.z
            sc[2] = s2[1];  // r.r
            sc[3] = zk0;    // p_k
            sc[4] = zk1;
        }
    }
    __syncthreads();
    double beta = sc[0], rz = sc[1], rr = sc[2], pk0 = sc[3], pk1 = sc[4];
    __syncthreads();
    const double bb = rr;
    int pit = 0, cur = 0;
    for (; pit < P.max_it; ++pit) {
        if (pit % 4 == 0 && !(rr > P.tol2 * bb)) break;
        const double* po = P.p[cur];
        double* pn = P.p[cur ^ 1];
        const Real* pro = P.pr[cur];
        Real* prn = P.pr[cur ^ 1];
        const Real betar = (Real)beta;
        // phase 1: p = z + beta p, q = S p (warp per camera row)
        {
            double pq = 0.0, kq0 = 0.0, kq1 = 0.0;
            for (int a = gw; a < P.nfc; a += nwarp) {
                // the row owner's own entries (lanes 0..5), loaded ahead of the products
                const int io = 6 * a + (lane < 6 ? lane : 0);
                const double zi = P.z[io], poi = po[io];
                const Real zri = P.zr[8 * a + (lane < 6 ? lane : 0)], pori = pro[8 * a + (lane < 6 ? lane : 0)];
                double h0 = 0.0, h1 = 0.0, x0 = 0.0, x1 = 0.0;
                if (P.nk && lane < 6) {
                    h0 = P.Hck[12LL * a + 2 * lane];
                    h1 = P.Hck[12LL * a + 2 * lane + 1];
                    x0 = P.Xak[12LL * a + 2 * lane];
                    x1 = P.Xak[12LL * a + 2 * lane + 1];
                }
                Real acc[6] = {Real(0), Real(0), Real(0), Real(0), Real(0), Real(0)};
                const int s1 = P.rs_off[a + 1];
                // two slots per lane per round (both slots' loads in flight together); the second
                // is a copy of the first with a zero direction where the row has no more slots
                for (int sl = P.rs_off[a] + lane; sl < s1; sl += 64) {
                    const bool two = sl + 32 < s1;
                    const int sl2 = two ? sl + 32 : sl;
                    const int bc = P.rs_col[sl], bc2 = P.rs_col[sl2];
                    Real sv[36], sv2[36];
                    load36(P.Sb + 36LL * sl, sv);
                    load36(P.Sb + 36LL * sl2, sv2);
                    Real pb[6], zb[6], pb2[6], zb2[6];
                    load6(P.zr + 8LL * bc, zb);
                    load6(pro + 8LL * bc, pb);
                    load6(P.zr + 8LL * bc2, zb2);
                    load6(pro + 8LL * bc2, pb2);
#pragma unroll
                    for (int j = 0; j < 6; ++j) {
                        pb[j] = zb[j] + betar * pb[j];
                        pb2[j] = two ? zb2[j] + betar * pb2[j] : Real(0);
                    }
#pragma unroll
                    for (int i = 0; i < 6; ++i)
#pragma unroll
                        for (int j = 0; j < 6; ++j) acc[i] += sv[6 * i + j] * pb[j];
#pragma unroll
                    for (int i = 0; i < 6; ++i)
#pragma unroll
                        for (int j = 0; j < 6; ++j) acc[i] += sv2[6 * i + j] * pb2[j];
                }
#pragma unroll
                for (int i = 0; i < 6; ++i)
#pragma unroll
                    for (int o = 16; o > 0; o >>= 1) acc[i] += __shfl_xor_sync(kFullG, acc[i], o);
                const Real qv = lane_value<6>(acc, lane);  // lanes 0..5: entry `lane` of the row
                if (lane < 6) {
                    const double c0 = h0 - x0, c1 = h1 - x1;
                    const double pv = zi + beta * poi;
                    const double qa = (double)qv + c0 * pk0 + c1 * pk1;
                    kq0 += c0 * pv;
                    kq1 += c1 * pv;
                    pn[6 * a + lane] = pv;
                    prn[8 * a + lane] = zri + betar * pori;
                    P.q[6 * a + lane] = qa;
                    pq += pv * qa;
                }
            }
            if (kthread) {
                pn[kb] = pk0;
                pn[kb + 1] = pk1;
            }
            mark(1);
            double three[3] = {pq, kq0, kq1};
            block_sum_w0<3>(three, mv_part);
        }
        grid.sync();
        mark(2);
        // phase 2: q_k, alpha; x += alpha p, r -= alpha q, z = M^-1 r; r.z and r.r partials
        {
            if (threadIdx.x < 32) {
                double s3[3] = {0.0, 0.0, 0.0};
                for (int i = lane; i < nb; i += 32) {
                    s3[0] += mv_part[3 * i];
                    s3[1] += mv_part[3 * i + 1];
                    s3[2] += mv_part[3 * i + 2];
                }
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) {
                    s3[0] += __shfl_down_sync(kFullG, s3[0], o);
                    s3[1] += __shfl_down_sync(kFullG, s3[1], o);
                    s3[2] += __shfl_down_sync(kFullG, s3[2], o);
                }
                if (lane == 0) {
                    double pq = s3[0], qk0 = 0.0, qk1 = 0.0;
                    if (P.nk) {
                        qk0 = P.skk[0] * pk0 + P.skk[1] * pk1 + s3[1];
                        qk1 = P.skk[1] * pk0 + P.skk[2] * pk1 + s3[2];
                        pq += pk0 * qk0 + pk1 * qk1;
                    }
                    sc[0] = pq != 0.0 ? rz / pq : 0.0;  // alpha
                    sc[1] = qk0;
                    sc[2] = qk1;
                }
            }
            __syncthreads();
            const double alpha = sc[0], qk0 = sc[1], qk1 = sc[2];
            __syncthreads();
            double rzn = 0.0, rrn = 0.0;
            for (int c = blockIdx.x + nb * wib; c < nchunk; c += nb * nwb) {
                const int a = 5 * c + grp;
                const bool act = grp < 5 && a < P.nfc;
                const int i = 6 * a + comp;
                double xv = 0.0, rv = 0.0, pv = 0.0, qv = 0.0;
                if (act) {
                    xv = P.x[i];
                    rv = P.r[i];
                    pv = pn[i];
                    qv = P.q[i];
                }
                xv += alpha * pv;
                rv -= alpha * qv;
                const double zv = apply_inv(a, act, rv);
                if (act) {
                    P.x[i] = xv;
                    P.r[i] = rv;
                    P.z[i] = zv;
                    P.zr[8 * a + comp] = (Real)zv;
                    rzn += rv * zv;
                    rrn += rv * rv;
                }
            }
            if (kthread) {
                const double xk0 = P.x[kb], xk1 = P.x[kb + 1], rk0 = P.r[kb], rk1 = P.r[kb + 1];
                const double r0 = rk0 - alpha * qk0, r1 = rk1 - alpha * qk1;
                double z0, z1;
                precond_k2(r0, r1, z0, z1);
                P.x[kb] = xk0 + alpha * pk0;
                P.x[kb + 1] = xk1 + alpha * pk1;
                P.r[kb] = r0;
                P.r[kb + 1] = r1;
                P.z[kb] = z0;
                P.z[kb + 1] = z1;
                rzn += r0 * z0 + r1 * z1;
                rrn += r0 * r0 + r1 * r1;
            }
            mark(3);
            double two[2] = {rzn, rrn};
            block_sum_w0<2>(two, rz_part);
        }
        grid.sync();
        mark(4);
        // beta, r.z, r.r and the next direction's k entries
        if (threadIdx.x < 32) {
            double zk0 = 0.0, zk1 = 0.0, pk0n = 0.0, pk1n = 0.0;
            if (P.nk && lane == 0) {
                zk0 = P.z[kb];
                zk1 = P.z[kb + 1];
                pk0n = pn[kb];
                pk1n = pn[kb + 1];
            }
            double s2[2] = {0.0, 0.0};
            for (int i = lane; i < nb; i += 32) {
                s2[0] += rz_part[2 * i];
                s2[1] += rz_part[2 * i + 1];
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                s2[0] += __shfl_down_sync(kFullG, s2[0], o);
                s2[1] += __shfl_down_sync(kFullG, s2[1], o);
            }
            if (lane == 0) {
                const double bn = rz != 0.0 ? s2[0] / rz : 0.0;
                sc[0] = bn;
                sc[1] = s2[0];
                sc[2] = s2[1];
                sc[3] = zk0 + bn * pk0n;
                sc[4] = zk1 + bn * pk1n;
            }
        }
        __syncthreads();
        beta = sc[0];
        rz = sc[1];
        rr = sc[2];
        pk0 = sc[3];
        pk1 = sc[4];
        __syncthreads();
        cur ^= 1;
        mark(0);
    }
    if (tid == 0) P.iters[0] = pit;
}

template <class Real>
__global__ void k_fold_intr(WinArgs<Real> A, WinDesc D, const Real* pt_b, double dk1, double dk2) {
    const CC c = grid_view();
    for (int p = c.gt; p < D.npt; p += c.CT) {
        if (A.pt_free[p] < 0) continue;
        Real b[12];
        Rec<Real>::load12(pt_b + 12LL * p, b);
        Real* lt = A.pt_lt + 12LL * p;
        lt[6] -= b[0] * (Real)dk1 + b[3] * (Real)dk2;
        lt[7] -= b[1] * (Real)dk1 + b[4] * (Real)dk2;
        lt[8] -= b[2] * (Real)dk1 + b[5] * (Real)dk2;
    }
}

// ---- host side ---------------------------------------------------------------------------

// Pair list storage: default-initialized (no zero fill of arrays of tens of millions of entries).
template <class T>
struct RawVec {
    std::unique_ptr<T[]> d;
    size_t n = 0;
    void resize(size_t k) {
        d.reset(new T[std::max<size_t>(k, 1)]);
        n = k;
    }
    T* data() { return d.get(); }
    const T* data() const { return d.get(); }
    size_t size() const { return n; }
    T& operator[](size_t i) { return d[i]; }
};

// Form of the reduced system a grid solve needs.
enum GridForm {
    kFormNone = 0,      // implicit PCG: S only as products with the per-edge records
    kFormCholesky = 1,  // lower blocks with pair lists, dense S, Cholesky work lists
    kFormBlocks = 2,    // lower blocks with pair lists, block rows of both triangles (explicit PCG)
};

struct GridHost {
    std::vector<int32_t> cam_list, item_off, fcam, boff, tfirst;
    std::vector<int32_t> tlast;  // per tile row I: the last tile row J with tfirst[J] <= I (S's extent)
    std::vector<int4> items;
    std::vector<int2> blocks;
    RawVec<int2> pairs;
    // Cholesky work per tile column K: panel tile rows and trailing tiles (I, J), K < J <= I
    std::vector<int32_t> pan_off, pan_row, tr_off, tr_skip;
    std::vector<int2> tr_ij;
    int max_col_work = 1;  // largest per-column count of panel tiles or trailing quarter items
    int max_npan = 0;      // largest per-column count of panel tiles
    // block rows of both triangles: row a's slots [rs_off[a], rs_off[a+1]) with their column
    // cameras rs_col in increasing order, its diagonal slot rs_dslot[a]; per lower block its slot
    // in its own row and the slot of the transposed block (-1 on the diagonal)
    std::vector<int32_t> rs_off, rs_col, rs_dslot;
    std::vector<int2> bslot;
    // work items of the Schur-block kernel: block, first and end pair, first item of the block
    std::vector<int4> sitems;
};

// Sum over points of k (k + 1) / 2 (k: free-camera observations of a free point): the pair count
// of the lower blocks, from the point offsets alone.
long long schur_pair_count(const HostWindow& h) {
    long long n = 0;
    for (int i = 0; i < h.npt; ++i) {
        if (h.pt_free[i] < 0) continue;
        long long k = 0;
        for (int e = h.pt_eoff[i]; e < h.pt_eoff[i + 1]; ++e) k += h.cam_free[h.edge_cam[e]] >= 0;
        n += k * (k + 1) / 2;
    }
    return n;
}

// The reduced system's structure for the given form.  Rows of the lower block structure are
// independent (row a's blocks and pairs come from camera a's edges alone), so they are built by
// row ranges on the host workers; every row is filled in the same order as a single pass would.
void build_grid_host(const HostWindow& h, GridHost& g, int form, HostPool* pool) {
    const int nfc = h.nfc;
    const char* verbose = getenv("NAVBA_VERBOSE");
    auto t0 = std::chrono::steady_clock::now();
    auto lap = [&](const char* what) {
        if (!verbose || verbose[0] != '1') return;
        const auto t1 = std::chrono::steady_clock::now();
        fprintf(stderr, "[navba grid] host %-14s %.2f ms\n", what, std::chrono::duration<double, std::milli>(t1 - t0).count());
        t0 = t1;
    };
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
    g.blocks.assign(1, make_int2(0, 0));
    g.boff.assign(2, 0);
    g.pairs.resize(1);
    g.pairs[0] = make_int2(0, 0);
    g.tfirst.assign(1, 0);
    g.tlast.assign(1, 0);
    g.pan_off.assign(2, 0);
    g.tr_off.assign(2, 0);
    g.tr_skip.assign(1, 0);
    g.pan_row.assign(1, 0);
    g.tr_ij.assign(1, make_int2(0, 0));
    g.max_col_work = 1;
    g.max_npan = 0;
    g.rs_off.assign(nfc + 1, 0);
    g.rs_col.assign(1, 0);
    g.rs_dslot.assign(std::max(1, nfc), 0);
    g.bslot.assign(1, make_int2(0, -1));
    g.sitems.assign(1, make_int4(0, 0, 0, 0));
    lap("camera lists");
    if (form == kFormNone) return;
    // row ranges on the workers (more ranges than workers: rows differ in cost)
    const int hw = std::max(1, (int)std::thread::hardware_concurrency());
    const int ntask = std::max(1, std::min(nfc, pool ? 4 * hw : 1));
    auto rows_of = [&](int t, int& a0, int& a1) {
        a0 = (int)((long long)nfc * t / ntask);
        a1 = (int)((long long)nfc * (t + 1) / ntask);
    };
    auto run = [&](const std::function<void(int)>& fn) {
        if (pool && ntask > 1)
            pool->run(ntask, fn);
        else
            for (int t = 0; t < ntask; ++t) fn(t);
    };
    std::vector<std::vector<int32_t>> rowcols(nfc);
    std::vector<int32_t> row_start(nfc + 1, 0);
    int nblk = 0;
    // NAVBA_GRID_HOST=rows takes the per-row passes at any size (they give the same lists)
    const char* hp = getenv("NAVBA_GRID_HOST");
    const bool by_rows = hp && !strcmp(hp, "rows");
    if (!by_rows && (size_t)nfc * nfc <= ((size_t)1 << 24)) {
        // Point-major passes over contiguous point ranges (sequential reads of each point's
        // observations), with a dense nfc x nfc map of the co-observing pairs.  Within a block
        // the pairs come in point order, then edge order: the same list the per-row passes build.
        const int npt = h.npt;
        const int T = std::max(1, std::min(pool ? hw : 1, npt / 4096));
        auto pts_of = [&](int t, int& i0, int& i1) {
            i0 = (int)((long long)npt * t / T);
            i1 = (int)((long long)npt * (t + 1) / T);
        };
        auto run_pts = [&](const std::function<void(int)>& fn) {
            if (pool && T > 1)
                pool->run(T, fn);
            else
                for (int t = 0; t < T; ++t) fn(t);
        };
        // every (e, f) pair of a free point with free cameras a = cam(e) >= b = cam(f)
        auto for_pairs = [&](int i, auto fn) {
            const int e0 = h.pt_eoff[i], e1 = h.pt_eoff[i + 1];
            for (int e = e0; e < e1; ++e) {
                const int a = h.cam_free[h.edge_cam[e]];
                if (a < 0) continue;
                for (int f = e0; f < e1; ++f) {
                    const int b = h.cam_free[h.edge_cam[f]];
                    if (b >= 0 && b <= a) fn(a, b, e, f);
                }
            }
        };
        // pass 1: the map of nonzero lower blocks (relaxed atomic flags: the same value from any task)
        std::vector<uint8_t> seen((size_t)nfc * nfc, 0);
        run_pts([&](int t) {
            int i0, i1;
            pts_of(t, i0, i1);
            for (int i = i0; i < i1; ++i) {
                if (h.pt_free[i] < 0) continue;
                for_pairs(i, [&](int a, int b, int, int) {
                    uint8_t* m = &seen[(size_t)a * nfc + b];
                    if (!__atomic_load_n(m, __ATOMIC_RELAXED)) __atomic_store_n(m, (uint8_t)1, __ATOMIC_RELAXED);
                });
            }
        });
        std::vector<int32_t> bidx((size_t)nfc * nfc, -1);
        for (int a = 0; a < nfc; ++a) {
            seen[(size_t)a * nfc + a] = 1;
            for (int b = 0; b <= a; ++b)
                if (seen[(size_t)a * nfc + b]) rowcols[a].push_back(b);
            row_start[a + 1] = row_start[a] + (int32_t)rowcols[a].size();
            for (size_t k = 0; k < rowcols[a].size(); ++k) bidx[(size_t)a * nfc + rowcols[a][k]] = row_start[a] + (int32_t)k;
        }
        nblk = row_start[nfc];
        g.blocks.resize(std::max(1, nblk));
        for (int a = 0; a < nfc; ++a)
            for (size_t k = 0; k < rowcols[a].size(); ++k) g.blocks[row_start[a] + k] = make_int2(a, rowcols[a][k]);
        // pass 2: pair counts per point range and block; the ranges' cursors in point order
        std::vector<int32_t> cnt((size_t)T * std::max(1, nblk), 0);
        run_pts([&](int t) {
            int i0, i1;
            pts_of(t, i0, i1);
            int32_t* c = cnt.data() + (size_t)t * nblk;
            for (int i = i0; i < i1; ++i) {
                if (h.pt_free[i] < 0) continue;
                for_pairs(i, [&](int a, int b, int, int) { c[bidx[(size_t)a * nfc + b]]++; });
            }
        });
        g.boff.assign(nblk + 1, 0);
        for (int k = 0; k < nblk; ++k) {
            int32_t sum = g.boff[k];
            for (int t = 0; t < T; ++t) {
                const int32_t n = cnt[(size_t)t * nblk + k];
                cnt[(size_t)t * nblk + k] = sum;  // now the range's cursor
                sum += n;
            }
            g.boff[k + 1] = sum;
        }
        if (g.boff.size() == 1) g.boff.push_back(0);
        lap("blocks");
        // pass 3: fill
        g.pairs.resize(std::max<size_t>(1, (size_t)g.boff[nblk]));
        g.pairs[0] = make_int2(0, 0);
        run_pts([&](int t) {
            int i0, i1;
            pts_of(t, i0, i1);
            int32_t* c = cnt.data() + (size_t)t * nblk;
            for (int i = i0; i < i1; ++i) {
                if (h.pt_free[i] < 0) continue;
                for_pairs(i, [&](int a, int b, int e, int f) { g.pairs[c[bidx[(size_t)a * nfc + b]]++] = make_int2(e, f); });
            }
        });
    } else {
        // pass 1, per row a: the columns b <= a of its nonzero blocks (sorted; a itself always) and
        // each block's pair count
        std::vector<std::vector<int32_t>> rowcnt(nfc);
        run([&](int t) {
            int a0, a1;
            rows_of(t, a0, a1);
            std::vector<int32_t> loc(nfc, -1), cols, cn, perm;
            for (int a = a0; a < a1; ++a) {
                cols.assign(1, a);
                cn.assign(1, 0);
                loc[a] = 0;
                for (int s = loff[a]; s < loff[a + 1]; ++s) {
                    const int i = h.edge_pt[g.cam_list[s]];
                    if (h.pt_free[i] < 0) continue;
                    for (int f = h.pt_eoff[i]; f < h.pt_eoff[i + 1]; ++f) {
                        const int b = h.cam_free[h.edge_cam[f]];
                        if (b < 0 || b > a) continue;
                        int k = loc[b];
                        if (k < 0) {
                            k = loc[b] = (int)cols.size();
                            cols.push_back(b);
                            cn.push_back(0);
                        }
                        cn[k]++;
                    }
                }
                perm.resize(cols.size());
                for (size_t k = 0; k < perm.size(); ++k) perm[k] = (int32_t)k;
                std::sort(perm.begin(), perm.end(), [&](int32_t x, int32_t y) { return cols[x] < cols[y]; });
                rowcols[a].resize(cols.size());
                rowcnt[a].resize(cols.size());
                for (size_t k = 0; k < perm.size(); ++k) {
                    rowcols[a][k] = cols[perm[k]];
                    rowcnt[a][k] = cn[perm[k]];
                }
                for (int b : cols) loc[b] = -1;
            }
        });
        for (int a = 0; a < nfc; ++a) row_start[a + 1] = row_start[a] + (int32_t)rowcols[a].size();
        nblk = row_start[nfc];
        g.blocks.resize(std::max(1, nblk));
        g.boff.assign(nblk + 1, 0);
        for (int a = 0; a < nfc; ++a)
            for (size_t k = 0; k < rowcols[a].size(); ++k) {
                const int blk = row_start[a] + (int)k;
                g.blocks[blk] = make_int2(a, rowcols[a][k]);
                g.boff[blk + 1] = g.boff[blk] + rowcnt[a][k];
            }
        if (g.boff.size() == 1) g.boff.push_back(0);
        lap("blocks");
        // pass 2, per row: the pairs of each block in camera-list (point) order
        g.pairs.resize(std::max<size_t>(1, (size_t)g.boff[nblk]));
        g.pairs[0] = make_int2(0, 0);
        run([&](int t) {
            int a0, a1;
            rows_of(t, a0, a1);
            std::vector<int32_t> loc(nfc, -1), cur;
            for (int a = a0; a < a1; ++a) {
                const auto& rc = rowcols[a];
                cur.resize(rc.size());
                for (size_t k = 0; k < rc.size(); ++k) {
                    loc[rc[k]] = (int32_t)k;
                    cur[k] = g.boff[row_start[a] + k];
                }
                for (int s = loff[a]; s < loff[a + 1]; ++s) {
                    const int e = g.cam_list[s];
                    const int i = h.edge_pt[e];
                    if (h.pt_free[i] < 0) continue;
                    for (int f = h.pt_eoff[i]; f < h.pt_eoff[i + 1]; ++f) {
                        const int b = h.cam_free[h.edge_cam[f]];
                        if (b >= 0 && b <= a) g.pairs[cur[loc[b]]++] = make_int2(e, f);
                    }
                }
                for (int b : rc) loc[b] = -1;
            }
        });
    }
    // work items: the explicit-PCG form splits the pair lists (large problems: the L2 window); the
    // Cholesky form keeps one item per block
    const int chunk = form == kFormBlocks ? kPairChunk : INT32_MAX;
    g.sitems.clear();
    for (int k = 0; k < nblk; ++k) {
        const int first = (int)g.sitems.size();
        const int p0 = g.boff[k], p1 = g.boff[k + 1];
        int q = p0;
        do {
            const int q1 = p1 - q > chunk ? q + chunk : p1;
            g.sitems.push_back(make_int4(k, q, q1, first));
            q = q1;
        } while (q < p1);
    }
    if (g.sitems.empty()) g.sitems.push_back(make_int4(0, 0, 0, 0));
    lap("pairs");
    if (form == kFormBlocks) {
        // row a: its lower columns (ending with a), then the columns c > a whose row holds a
        std::vector<int32_t> upc(nfc, 0);
        for (int a = 0; a < nfc; ++a)
            for (int b : rowcols[a])
                if (b < a) upc[b]++;
        for (int a = 0; a < nfc; ++a) g.rs_off[a + 1] = g.rs_off[a] + (int32_t)rowcols[a].size() + upc[a];
        g.rs_col.assign(std::max(1, g.rs_off[nfc]), 0);
        g.bslot.resize(std::max(1, nblk));
        std::vector<int32_t> ucur(nfc);
        for (int a = 0; a < nfc; ++a) {
            const int nl = (int)rowcols[a].size();
            ucur[a] = g.rs_off[a] + nl;
            g.rs_dslot[a] = g.rs_off[a] + nl - 1;
            for (int k = 0; k < nl; ++k) g.rs_col[g.rs_off[a] + k] = rowcols[a][k];
        }
        for (int a = 0; a < nfc; ++a)  // increasing a: the upper columns of each row come sorted
            for (size_t k = 0; k < rowcols[a].size(); ++k) {
                const int b = rowcols[a][k];
                int up = -1;
                if (b < a) {
                    up = ucur[b]++;
                    g.rs_col[up] = a;
                }
                g.bslot[row_start[a] + k] = make_int2(g.rs_off[a] + (int)k, up);
            }
        lap("block rows");
        if (verbose && verbose[0] == '1') {
            int longest = 0;
            for (int a = 0; a < nfc; ++a) longest = std::max(longest, g.rs_off[a + 1] - g.rs_off[a]);
            fprintf(stderr, "[navba grid] explicit S: %d cameras, %d lower blocks, %d slots (longest row %d), %zu pairs\n",
                    nfc, nblk, g.rs_off[nfc], longest, g.pairs.size());
        }
        return;
    }
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
    // the symmetric envelope's extent: row i of the mirrored S is zero beyond tile tlast[i / 32]
    g.tlast.assign(std::max(1, nt), 0);
    for (int J = 0; J < nt; ++J)
        for (int I = g.tfirst[J]; I <= J; ++I) g.tlast[I] = std::max(g.tlast[I], J);
    g.pan_off.assign(nt + 1, 0);
    g.tr_off.assign(nt + 1, 0);
    g.pan_row.clear();
    g.tr_ij.clear();
    // per tile column K: its panel rows rows(K) and the trailing tiles it updates (pairs of rows(K))
    g.max_col_work = 1;
    g.max_npan = 0;
    g.tr_skip.assign(std::max(1, nt), 0);
    for (int K = 0; K < nt; ++K) {
        std::vector<int32_t> rows;
        for (int I = K + 1; I < nt; ++I)
            if (g.tfirst[I] <= K) rows.push_back(I);
        for (int I : rows) g.pan_row.push_back(I);
        for (size_t y = 0; y < rows.size(); ++y)  // by column J = rows[y]
            for (size_t x = y; x < rows.size(); ++x) g.tr_ij.push_back(make_int2(rows[x], rows[y]));
        // left out when the FP32 factorization applies this column's update one phase later: the
        // tiles of column K + 1, which their panel blocks update themselves
        g.tr_skip[K] = (!rows.empty() && rows[0] == K + 1) ? (int32_t)rows.size() : 0;
        g.pan_off[K + 1] = (int32_t)g.pan_row.size();
        g.tr_off[K + 1] = (int32_t)g.tr_ij.size();
        g.max_col_work = std::max(g.max_col_work, (int)rows.size() + 4 * (g.tr_off[K + 1] - g.tr_off[K]));
        g.max_npan = std::max(g.max_npan, (int)rows.size());
    }
    if (g.pan_row.empty()) g.pan_row.push_back(0);
    if (g.tr_ij.empty()) g.tr_ij.push_back(make_int2(0, 0));
}

// Device buffers of one grid solve, carved in order from the workspace's slab (256-byte aligned)
// while it has room, else allocated one by one.  At the end of the call the slab grows to what
// the call needed, so a repeated solve of the same size allocates nothing (the per-buffer
// allocations and frees were ~1 ms of a 20 ms solve of 200 cameras; a free also waits for the
// device).  The buffers' contents are not initialized either way.
struct GridDev {
    GridWorkspace* ws = nullptr;  // non-null while this call holds the workspace
    bool use_slab = false;
    char* base = nullptr;
    size_t cap = 0, off = 0, need = 0;
    std::vector<void*> ptrs;
    cudaError_t err = cudaSuccess;
    explicit GridDev(GridWorkspace* w) {
        if (!w || w->busy) return;
        ws = w;
        ws->busy = true;
        const char* v = getenv("NAVBA_GRID_WORKSPACE");
        use_slab = !(v && v[0] == '0');
        if (use_slab) {
            base = static_cast<char*>(ws->slab.p);
            cap = ws->slab.cap;
        }
    }
    template <class T>
    T* alloc(size_t n) {
        if (err != cudaSuccess) return nullptr;
        const size_t bytes = (std::max<size_t>(n, 1) * sizeof(T) + 255) & ~size_t(255);
        need += bytes;
        if (base && off + bytes <= cap) {
            void* p = base + off;
            off += bytes;
            return static_cast<T*>(p);
        }
        void* p = nullptr;
        err = cudaMalloc(&p, bytes);
        if (err == cudaSuccess) ptrs.push_back(p);
        return static_cast<T*>(p);
    }
    // page-locked host memory of at least `bytes` from the workspace (grown on demand), or nullptr
    void* pinned(size_t bytes) {
        if (!ws) return nullptr;
        if (ws->pinned_cap < bytes) {
            if (ws->pinned) cudaFreeHost(ws->pinned);
            ws->pinned = nullptr;
            ws->pinned_cap = 0;
            if (cudaMallocHost(&ws->pinned, bytes) != cudaSuccess) {
                ws->pinned = nullptr;
                cudaGetLastError();
                return nullptr;
            }
            ws->pinned_cap = bytes;
        }
        return ws->pinned;
    }
    ~GridDev() {
        for (void* p : ptrs) cudaFree(p);
        if (!ws) return;
        if (use_slab && need > ws->slab.cap) {
            // a failed allocation leaves no slab: the next call allocates buffer by buffer
            cudaError_t e = cudaSuccess;
            ws->slab.release();
            if (!ws->slab.get(need, &e)) cudaGetLastError();
        }
        ws->busy = false;
    }
};

template <class T>
cudaError_t up(T* d, const std::vector<T>& h, cudaStream_t s) {
    if (h.empty()) return cudaSuccess;
    return cudaMemcpyAsync(d, h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice, s);
}

template <class T>
cudaError_t up(T* d, const RawVec<T>& h, cudaStream_t s) {
    if (!h.size()) return cudaSuccess;
    return cudaMemcpyAsync(d, h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice, s);
}

template <class Real>
cudaError_t grid_solve_typed(const HostWindow& h, const LmOptions& lm, const Intr& intr, cudaStream_t st,
                             HostPool* pool, GridWorkspace* ws, GridResult& out, double debug_lambda,
                             std::vector<double>* debug_S, GridVjp* vjp) {
    const auto tg0 = std::chrono::steady_clock::now();
    auto ms_from = [](std::chrono::steady_clock::time_point a) {
        return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - a).count();
    };
    const bool pcg = lm.solver == NAV_BA_SOLVER_PCG && !debug_S;
    // PCG over the explicit block-sparse S unless its pair lists would be long against the
    // observations (points seen by very many cameras): then the products go through the
    // per-observation records (implicit S).  NAVBA_PCG_FORM=explicit|implicit fixes the form.
    // (pair lists are indexed by int32 offsets: beyond 2^30 pairs the implicit form is taken)
    bool pcg_x = false;
    if (pcg && !vjp) {
        const long long npairs = schur_pair_count(h);
        const char* f = getenv("NAVBA_PCG_FORM");
        if (f && !strcmp(f, "implicit"))
            pcg_x = false;
        else if (f && !strcmp(f, "explicit"))
            pcg_x = true;
        else
            pcg_x = npairs <= 24LL * std::max(1, h.ne);
        pcg_x = pcg_x && npairs < (1LL << 30);
    }
    GridHost g;
    build_grid_host(h, g, (!pcg || vjp != nullptr) ? kFormCholesky : (pcg_x ? kFormBlocks : kFormNone), pool);
    const double t_host = ms_from(tg0);
    const int nc = h.ncam, np = h.npt, ne = h.ne, nfc = h.nfc;
    const int m = 6 * nfc;
    GridDev dv(ws);
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
    Real* d_w = sizeof(Real) == 8 ? dv.alloc<Real>(rec * ne) : nullptr;  // FP64 form: stored W
    Real* d_a = dv.alloc<Real>(rec * ne);
    Real* d_camr0 = dv.alloc<Real>(12LL * nc);
    Real* d_camr1 = dv.alloc<Real>(12LL * nc);
    double* d_camd = dv.alloc<double>(12LL * nc);
    // mixed form, PCG: each edge's residual from the FP64 cost pass of state 0 / 1 (what the mixed
    // linearization uses instead of its FP32 residuals).  The Cholesky path keeps FP32 residuals: with
    // exact gradients its damping falls to where the FP32 factorization fails and the FP64 one runs
    // instead (200-camera grid: 45 -> 71 ms, final costs 2e-8 -> 1e-10 of the FP64 form's)
    Real* d_ep[2] = {nullptr, nullptr};
    if (sizeof(Real) == 4 && lm.solver == NAV_BA_SOLVER_PCG && !debug_S) {
        d_ep[0] = dv.alloc<Real>(2LL * std::max(1, ne));
        d_ep[1] = dv.alloc<Real>(2LL * std::max(1, ne));
    }
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
    int32_t* d_tlast = dv.alloc<int32_t>(std::max<size_t>(1, g.tlast.size()));
    int32_t* d_pan_off = dv.alloc<int32_t>(g.pan_off.size());
    int32_t* d_pan_row = dv.alloc<int32_t>(g.pan_row.size());
    int32_t* d_tr_off = dv.alloc<int32_t>(g.tr_off.size());
    int32_t* d_tr_skip = dv.alloc<int32_t>(g.tr_skip.size());
    int2* d_tr_ij = dv.alloc<int2>(g.tr_ij.size());
    const int nk = (lm.optimize_k && intr.model == 1) ? 2 : 0;
    const int mt = m + nk;
    double* d_S = dv.alloc<double>(pcg ? 1 : (size_t)std::max(1, m) * std::max(1, m));
    // mixed form, Cholesky path (not the differentiable solve, which is FP64): the FP32 factor of S
    const bool mixed_chol = sizeof(Real) == 4 && !pcg && !vjp;
    float* d_S32 = mixed_chol ? dv.alloc<float>((size_t)std::max(1, m) * std::max(1, m)) : nullptr;
    float* d_rinv32 = mixed_chol ? dv.alloc<float>(std::max(1, m)) : nullptr;
    // the panel tiles transposed, for the forward solves (Cholesky path only)
    const size_t lt_elems = (!pcg || vjp != nullptr) ? g.pan_row.size() * (size_t)(kTile * kTile) : 1;
    const size_t di_elems = (!pcg || vjp != nullptr) ? (size_t)std::max(1, (m + kTile - 1) / kTile) * 2 * kTile * kTile : 1;
    float* d_LT32 = mixed_chol ? dv.alloc<float>(lt_elems) : nullptr;
    float* d_LN32 = mixed_chol ? dv.alloc<float>(lt_elems) : nullptr;
    float* d_DI32 = mixed_chol ? dv.alloc<float>(di_elems) : nullptr;
    double* d_LT = dv.alloc<double>(lt_elems);
    double* d_LN = dv.alloc<double>(lt_elems);
    double* d_DI = dv.alloc<double>(di_elems);
    float* d_x32 = mixed_chol ? dv.alloc<float>(std::max(1, m)) : nullptr;
    float* d_y32 = mixed_chol ? dv.alloc<float>(std::max(1, m)) : nullptr;
    double* d_bs = dv.alloc<double>(std::max(1, mt));
    double* d_rinv = dv.alloc<double>(std::max(1, m));
    int32_t* d_ok = dv.alloc<int32_t>(1);
    // the item-ordered Schur kernel's work counter, the factorization's failure flag and the
    // Schur blocks' item counts, zeroed together
    int32_t* d_flags = dv.alloc<int32_t>(2 + g.blocks.size());
    int32_t* d_next = d_flags;
    int32_t* d_fail = d_flags + 1;
    const int n_sitems = (int)g.sitems.size();
    int4* d_sitems = dv.alloc<int4>(g.sitems.size());
    int32_t* d_sdone = d_flags + 2;
    Real* d_spart = dv.alloc<Real>(48LL * n_sitems);
    const int TB = 256;
    const int nsm_blocks = 152 * 4;
    const int pblocks = std::max(1, std::min(nsm_blocks, (np + TB - 1) / TB));
    const int cblocks = std::max(1, (nc + TB - 1) / TB);
    const int ucblocks = std::max(1, (nc + 31) / 32);  // the trial's camera update: 32 cameras per block
    const int rblocks = (nfc * 27 + TB - 1) / TB;  // partials of the camera blocks' maxima
    const int npart = std::max(5 * pblocks, std::max(cblocks, pblocks + rblocks + 1));
    double* d_part = dv.alloc<double>(npart);
    // a damping trial's partial sums, read back together at its end: point blocks that failed,
    // the model decrease's camera and point terms, the trial cost
    double* d_tpart = dv.alloc<double>(3LL * pblocks + ucblocks);
    // PCG and distortion buffers
    const int n_items = (int)g.items.size();
    Real* d_kp = nk ? dv.alloc<Real>(12LL * np) : nullptr;
    Real* d_pb = nk ? dv.alloc<Real>(12LL * np) : nullptr;
    double* d_hpart = nk ? dv.alloc<double>(12LL * n_items) : nullptr;
    double* d_Hck = dv.alloc<double>(12LL * std::max(1, nfc));
    const bool pcg_i = pcg && !pcg_x;  // implicit S
    Real* d_t2 = pcg_i ? dv.alloc<Real>(4LL * np) : nullptr;
    double* d_aat = pcg_i ? dv.alloc<double>(28LL * std::max(1, nfc)) : nullptr;
    double* d_pc = pcg ? dv.alloc<double>(28LL * std::max(1, nfc)) : nullptr;
    double* d_pcinv = pcg ? dv.alloc<double>(36LL * std::max(1, nfc)) : nullptr;
    double* d_camp = pcg_i ? dv.alloc<double>(8LL * n_items) : nullptr;
    double* d_vec = pcg ? dv.alloc<double>(6LL * std::max(1, mt) + 8) : nullptr;
    // explicit S: block rows, slots of the lower blocks, camera-k coupling
    const int nslot = pcg_x ? g.rs_off[nfc] : 0;
    Real* d_Sb = pcg_x ? dv.alloc<Real>(36LL * std::max(1, nslot)) : nullptr;
    int32_t* d_rs_off = pcg_x ? dv.alloc<int32_t>(g.rs_off.size()) : nullptr;
    int32_t* d_rs_col = pcg_x ? dv.alloc<int32_t>(g.rs_col.size()) : nullptr;
    int32_t* d_rs_dslot = pcg_x ? dv.alloc<int32_t>(g.rs_dslot.size()) : nullptr;
    int2* d_bslot = pcg_x ? dv.alloc<int2>(g.bslot.size()) : nullptr;
    double* d_xak = (pcg_x && nk) ? dv.alloc<double>(12LL * std::max(1, nfc)) : nullptr;
    Real* d_zpr = pcg_x ? dv.alloc<Real>(24LL * std::max(1, nfc)) : nullptr;  // z, p, p in Real (8 per camera)
    double* d_kvals = dv.alloc<double>(8);  // [0..2] H_kk + lambda-free, [3..5] pk (2x2 Cholesky)
    // tape of the accepted steps (state before each step) and the backward's vectors
    const int tape_cap = vjp ? (vjp->replay ? (int)vjp->lambdas.size() : lm.iterations) : 0;
    CamState* d_tape_c = vjp ? dv.alloc<CamState>((size_t)std::max(1, tape_cap) * nc) : nullptr;
    double* d_tape_x = vjp ? dv.alloc<double>((size_t)std::max(1, tape_cap) * 4 * np) : nullptr;
    const bool bwd = vjp && vjp->backward;
    const int nfc1 = std::max(1, nfc);
    double* d_cb[2] = {bwd ? dv.alloc<double>(6LL * nfc1) : nullptr, bwd ? dv.alloc<double>(6LL * nfc1) : nullptr};
    double* d_rc = bwd ? dv.alloc<double>(6LL * nfc1) : nullptr;
    double* d_uc = bwd ? dv.alloc<double>(6LL * nfc1) : nullptr;
    double* d_ctmp = bwd ? dv.alloc<double>(6LL * nfc1) : nullptr;
    double* d_pbar = bwd ? dv.alloc<double>(4LL * np) : nullptr;
    double* d_up = bwd ? dv.alloc<double>(4LL * np) : nullptr;
    double* d_dp = bwd ? dv.alloc<double>(4LL * np) : nullptr;
    double* d_tr = bwd ? dv.alloc<double>(4LL * np) : nullptr;
    double* d_eadj = bwd ? dv.alloc<double>(8LL * ne) : nullptr;  // per-edge camera adjoints
    double* d_uvbar = bwd ? dv.alloc<double>(2LL * ne) : nullptr;
    double* d_ipart = bwd ? dv.alloc<double>(8LL * g.items.size()) : nullptr;
    double* d_posebar = (bwd && vjp->pose_bar) ? dv.alloc<double>(12LL * nc) : nullptr;
    double* d_ptbar = (bwd && vjp->point_bar) ? dv.alloc<double>(3LL * np) : nullptr;
    // PCG: structure-of-arrays copies of A (point-major, camera-major) and the camera list's points
    const int ncl = (int)g.cam_list.size();
    Real* d_apm = pcg_i ? dv.alloc<Real>(18LL * ne) : nullptr;
    Real* d_acm = pcg_i ? dv.alloc<Real>(18LL * ncl) : nullptr;
    int32_t* d_cmpt = pcg_i ? dv.alloc<int32_t>(ncl) : nullptr;
    float* d_pf = (pcg_i && sizeof(Real) == 4) ? dv.alloc<float>(6LL * nfc1) : nullptr;
    // cooperative PCG grid: every block resident (the occupancy bound of the kernel)
    int pcg_grid = 1;
    if (pcg) {
        int dev = 0, nsm = 0, bps = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
        if (pcg_x) {
            // enough warps for one camera row each, within what is resident
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, k_pcg_explicit<Real>, 256, 0);
            pcg_grid = std::max(1, std::min(nsm * std::max(1, std::min(bps, 4)), (nfc + 7) / 8));
        } else {
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, k_pcg_solve<Real>, 256, 0);
            pcg_grid = std::max(1, nsm * std::max(1, std::min(bps, 4)));
        }
    }
    double* d_ppart = pcg ? dv.alloc<double>(7LL * pcg_grid) : nullptr;
    int32_t* d_pit = pcg ? dv.alloc<int32_t>(1) : nullptr;
    const char* ptv = getenv("NAVBA_PHASE_TIMING");
    // NAVBA_PHASE_TIMING=1: block 0's cycles per phase of the PCG kernel or of the factorization
    unsigned long long* d_phase = ptv && ptv[0] == '1' ? dv.alloc<unsigned long long>(5) : nullptr;
    if (dv.err != cudaSuccess) return dv.err;
    if (d_phase) cudaMemsetAsync(d_phase, 0, 5 * sizeof(unsigned long long), st);
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
    chk(up(d_sitems, g.sitems, st));
    chk(up(d_tfirst, g.tfirst, st));
    chk(up(d_tlast, g.tlast, st));
    chk(up(d_pan_off, g.pan_off, st));
    chk(up(d_pan_row, g.pan_row, st));
    chk(up(d_tr_off, g.tr_off, st));
    chk(up(d_tr_skip, g.tr_skip, st));
    chk(up(d_tr_ij, g.tr_ij, st));
    if (pcg_x) {
        chk(up(d_rs_off, g.rs_off, st));
        chk(up(d_rs_col, g.rs_col, st));
        chk(up(d_rs_dslot, g.rs_dslot, st));
        chk(up(d_bslot, g.bslot, st));
    }
    std::vector<int32_t> cm_pt;
    if (pcg_i) {
        cm_pt.resize(ncl);
        for (int sl = 0; sl < ncl; ++sl) {
            const int pt = h.edge_pt[g.cam_list[sl]];
            cm_pt[sl] = h.pt_free[pt] >= 0 ? pt : -1;
        }
        chk(up(d_cmpt, cm_pt, st));
    }
    if (d_posebar) chk(cudaMemcpyAsync(d_posebar, vjp->pose_bar, sizeof(double) * 12 * nc, cudaMemcpyHostToDevice, st));
    if (d_ptbar) chk(cudaMemcpyAsync(d_ptbar, vjp->point_bar, sizeof(double) * 3 * np, cudaMemcpyHostToDevice, st));
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
    (void)mixed;
    double kcur[2] = {intr.k1, intr.k2};  // current shared distortion (free when nk == 2)
    double Kk[3] = {0, 0, 0}, gk[2] = {0, 0};
    int pcg_total = 0;
    // read-back buffers, page-locked when the workspace gives them (copies then run as the
    // stream's work; from pageable memory each copy waits for the device on its own): partial
    // sums, the linearization's maxima, a trial's partials, the shared-distortion step, flags
    const size_t ntp = 3LL * pblocks + ucblocks;
    const size_t nhost = 2 * (size_t)npart + ntp + 4;
    std::vector<double> hfallback;
    double* hpart = static_cast<double*>(dv.pinned(sizeof(double) * nhost));
    if (!hpart) {
        hfallback.assign(nhost, 0.0);
        hpart = hfallback.data();
    }
    double* hlin = hpart + npart;
    double* hpart_trial = hlin + npart;
    double* hdk = hpart_trial + ntp;
    int32_t* hflag = reinterpret_cast<int32_t*>(hdk + 2);  // [0] a pivot flag, [1] CG iterations, [2] 1
    hflag[2] = 1;  // the value a pivot flag is reset to
    auto sum_part = [&](int n, bool mx) -> double {
        if (e != cudaSuccess) return 0.0;
        e = cudaMemcpyAsync(hpart, d_part, sizeof(double) * n, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        double s = 0.0;
        for (int k = 0; k < n; ++k) s = mx ? std::max(s, hpart[k]) : s + hpart[k];
        return s;
    };
    auto cost_of = [&](int buf, bool fp64) -> double {
        if (fp64 && mixed) {
            k_cams_real<double><<<cblocks, TB, 0, st>>>(cams[buf], nc, d_camd);
            k_cost<double, Real><<<pblocks, TB, 0, st>>>(A, D, d_camd, A.x[buf], d_part, d_ep[buf]);
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
    chk(cudaStreamSynchronize(st));
    const double t_setup = ms_from(tg0);
    struct LoopTimer {
        std::chrono::steady_clock::time_point t0;
        double host, setup;
        double (*ms)(std::chrono::steady_clock::time_point);
        unsigned long long* phase;
        cudaStream_t st;
        int explicit_s;
        ~LoopTimer() {
            const char* v = getenv("NAVBA_VERBOSE");
            if (v && v[0] == '1')
                fprintf(stderr, "[navba grid] host structure %.2f ms, allocation + upload %.2f ms, LM loop %.2f ms\n", host,
                        setup - host, ms(t0));
            unsigned long long cyc[5] = {0, 0, 0, 0, 0};
            if (phase && cudaMemcpyAsync(cyc, phase, sizeof(cyc), cudaMemcpyDeviceToHost, st) == cudaSuccess &&
                cudaStreamSynchronize(st) == cudaSuccess) {
                static const char* names[3][5] = {{"point t2", "camera items", "S p", "x/r update", "p update"},
                                                  {"beta sums", "S p (own)", "S p (sync)", "x/r (own)", "x/r (sync)"},
                                                  {"diagonal", "panels", "trailing", "grid sync", "inverses"}};
                double tot = 0;
                for (int k = 0; k < 5; ++k) tot += (double)cyc[k];
                for (int k = 0; k < 5; ++k)
                    fprintf(stderr, "[navba grid] %s phase %-13s %14llu cycles %5.1f%%\n",
                            explicit_s == 2 ? "factorization" : "pcg", names[explicit_s][k], cyc[k],
                            tot > 0 ? 100.0 * cyc[k] / tot : 0.0);
            }
        }
    } loop_timer{std::chrono::steady_clock::now(), t_host, t_setup, +[](std::chrono::steady_clock::time_point a) {
                     return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - a).count();
                 }, d_phase, st, pcg ? (pcg_x ? 1 : 0) : 2};
    int cur = 0;
    // NAVBA_VERBOSE=2: one line per damping trial (damping, outcome, CG iterations)
    const char* vtrial = getenv("NAVBA_VERBOSE");
    const bool trial_log = vtrial && vtrial[0] == '2';
    // costs (initial, every trial) are evaluated in FP64 in both forms: they drive the gain ratio
    double chi = cost_of(0, true);
    out.initial_cost = chi;
    auto sum_parts = [&](int nblocks, int nval, double* outv) {
        if (e != cudaSuccess) return;
        e = cudaMemcpyAsync(hpart, d_part, sizeof(double) * nblocks * nval, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        for (int k = 0; k < nval; ++k) outv[k] = 0.0;
        for (int bI = 0; bI < nblocks; ++bI)
            for (int k = 0; k < nval; ++k) outv[k] += hpart[(size_t)nval * bI + k];
    };
    const int iblocks = std::max(1, std::min(nsm_blocks, (n_items * 32 + TB - 1) / TB));
    // linearization at state c: V_p, g_p (point-major), U_a, g_a (camera-major).  The max |diag|
    // of the point and camera blocks (g2o's initial damping; the mixed form's FP32 resolution) is
    // copied back behind an event and waited for only where it is used (lin_maxima), so the
    // device goes on with the trial's kernels meanwhile.
    cudaEvent_t ev_lin = nullptr;
    chk(cudaEventCreateWithFlags(&ev_lin, cudaEventDisableTiming));
    struct EventGuard {
        cudaEvent_t ev;
        ~EventGuard() {
            if (ev) cudaEventDestroy(ev);
        }
    } ev_lin_guard{ev_lin};
    auto linearize = [&](int c) {
        k_lin_points<Real><<<pblocks, TB, 0, st>>>(A, D, camr[c], A.x[c], d_part);
        if (nfc > 0) {
            k_lin_cams<Real><<<iblocks, TB, 0, st>>>(A, d_items, n_items, d_list, d_fcam, camr[c], A.x[c], d_upart);
            k_reduce_cams<<<rblocks, TB, 0, st>>>(d_upart, d_item_off, nfc, d_U, d_part + pblocks);
        }
        chk(cudaGetLastError());
        chk(cudaMemcpyAsync(hlin, d_part, sizeof(double) * (pblocks + (nfc > 0 ? rblocks : 0)), cudaMemcpyDeviceToHost,
                            st));
        chk(cudaEventRecord(ev_lin, st));
    };
    auto lin_maxima = [&](double& mxp, double& mxc) {
        if (e == cudaSuccess) e = cudaEventSynchronize(ev_lin);
        mxp = mxc = 0.0;
        if (e != cudaSuccess) return;
        for (int k = 0; k < pblocks; ++k) mxp = std::max(mxp, hlin[k]);
        for (int k = 0; nfc > 0 && k < rblocks; ++k) mxc = std::max(mxc, hlin[pblocks + k]);
    };
    // dense reduced system S = U + lam I - sum A A^T (lower part) and b'; the mixed form's FP32
    // copy (lower part) and the upper mirror of S with it.  The factorization's failure flag is
    // zeroed with the Schur kernel's counters.
    auto assemble_S = [&](double lam) {
        chk(cudaMemsetAsync(d_S, 0, sizeof(double) * (size_t)m * m, st));
        if (mixed_chol) chk(cudaMemsetAsync(d_S32, 0, sizeof(float) * (size_t)m * m, st));
        chk(cudaMemsetAsync(d_flags, 0, sizeof(int32_t) * (2 + g.blocks.size()), st));
        k_schur_blocks<Real><<<std::max(1, std::min(nsm_blocks, (n_sitems * 32 + TB - 1) / TB)), TB, 0, st>>>(
            A, d_blocks, d_boff, d_sitems, n_sitems, d_pairs, d_U, lam, d_S, m, d_bs, (Real*)nullptr, nullptr, d_next,
            d_sdone, d_spart, INT32_MAX, mixed_chol ? d_S32 : nullptr);
        chk(cudaGetLastError());
    };
    // Cholesky of S in place (cooperative, whole GPU); false if S is not positive definite
    int chol_grid = 1;
    {
        int dev = 0, nsm = 0, bps = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
        int bps32 = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, k_cholesky_coop<double>, 256, 0);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps32, k_cholesky_coop<float>, 256, 0);
        bps = std::min(bps, bps32);
        chol_grid = std::max(1, std::min(nsm * std::max(1, std::min(bps, 2)), g.max_col_work));
    }
    // defer: the failure flag (d_fail) is left for the trial's read-back instead of read here;
    // reset: zero the flag first (a factorization after another one; assemble_S zeroes it)
    auto factor_S = [&](bool defer = false, bool reset = false) -> bool {
        if (reset) chk(cudaMemsetAsync(d_fail, 0, sizeof(int32_t), st));
        double* Sp = d_S;
        int mm = m;
        const int32_t* tf = d_tfirst;
        const int32_t* po = d_pan_off;
        const int32_t* pr = d_pan_row;
        const int32_t* to = d_tr_off;
        const int32_t* tsk = d_tr_skip;
        const int2* tij = d_tr_ij;
        double* ri = d_rinv;
        double* ltp = d_LT;
        double* lnp = d_LN;
        double* dip = d_DI;
        int32_t* okp = d_fail;
        unsigned long long* cph = d_phase;
        void* kargs[] = {&Sp, &mm, &tf, &po, &pr, &to, &tsk, &tij, &ri, &ltp, &lnp, &dip, &okp, &cph};
        chk(cudaLaunchCooperativeKernel((const void*)k_cholesky_coop<double>, dim3(chol_grid), dim3(256), kargs, 0, st));
        if (defer) return e == cudaSuccess;
        chk(cudaMemcpyAsync(hflag, d_fail, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
        chk(cudaStreamSynchronize(st));
        return e == cudaSuccess && hflag[0] == 0;
    };
    // Mixed form: S x = b (x into d_bs) with the Cholesky factor of S rounded to FP32 and one FP64
    // refinement step (r = b - S x0 over the FP64 S, then the FP32 factor's solution of r added).
    // S's entries are FP32 sums already, so the FP32 factor's error is of the order of S's own; the
    // refinement step removes it.  A pivot that is not positive in FP32:
    // - at a damping below kF32Resolution of the largest Hessian diagonal entry ends the trial as a
    //   system that is not positive definite does (the damping grows; the flag is read with the
    //   trial's sums): the rounding of S, whose point blocks' (V + lambda I)^-1 are then large, is
    //   larger than the damping that makes it definite, and the FP64 factorization of the same S
    //   fails as well (measured on the 200-camera grid: every such attempt failed; raising only the
    //   FP32 factorization's diagonal, up to 64x the damping, did not make it definite either);
    // - above it, falls back to the FP64 factorization, and so do later trials at up to 4x the
    //   damping of the last failure (the failed attempt is not repeated).
    // Returns false if S is not positive definite.
    constexpr double kF32Resolution = 1e-6;
    double f32_fail_lambda = -1.0;
    // deferred: set when the FP32 pivot flag is left for the trial's read-back (no FP64 fallback
    // at this damping, so nothing waits on it)
    auto solve_S_mixed = [&](double lam, double maxdiag, bool& deferred) -> bool {
        const bool f64_useful = lam >= kF32Resolution * maxdiag;
        deferred = false;
        if (f64_useful && f32_fail_lambda > 0.0 && lam <= 4.0 * f32_fail_lambda) {
            if (!factor_S()) return false;
            chk(chol_solve(d_LT, d_LN, d_DI, m, d_pan_off, d_pan_row, d_bs, g.max_npan, st));
            return true;
        }
        float* Sp = d_S32;
        int mm = m;
        const int32_t* tf = d_tfirst;
        const int32_t* po = d_pan_off;
        const int32_t* pr = d_pan_row;
        const int32_t* to = d_tr_off;
        const int32_t* tsk = d_tr_skip;
        const int2* tij = d_tr_ij;
        float* ri = d_rinv32;
        float* ltp = d_LT32;
        float* lnp = d_LN32;
        float* dip = d_DI32;
        int32_t* okp = d_fail;
        unsigned long long* cph = d_phase;
        void* kargs[] = {&Sp, &mm, &tf, &po, &pr, &to, &tsk, &tij, &ri, &ltp, &lnp, &dip, &okp, &cph};
        chk(cudaLaunchCooperativeKernel((const void*)k_cholesky_coop<float>, dim3(chol_grid), dim3(256), kargs, 0, st));
        int32_t okh = 1;
        if (f64_useful) {
            chk(cudaMemcpyAsync(hflag, d_fail, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
            chk(cudaStreamSynchronize(st));
            okh = hflag[0] == 0;
        } else {
            deferred = true;
        }
        if (e != cudaSuccess) return false;
        if (!okh) {
            const char* vb = getenv("NAVBA_VERBOSE");
            if (vb && vb[0] == '1')
                fprintf(stderr, "[navba grid] FP32 factor: non-positive pivot, %s\n",
                        f64_useful ? "FP64 factor instead" : "trial rejected");
            if (!f64_useful) return false;
            f32_fail_lambda = std::max(f32_fail_lambda, lam);
            if (!factor_S(false, true)) return false;
            chk(chol_solve(d_LT, d_LN, d_DI, m, d_pan_off, d_pan_row, d_bs, g.max_npan, st));
            return true;
        }
        // x0 = S32^-1 (float)b; y = S32^-1 (b - S x0); b <- x0 + y (the solves convert on load and store)
        chk(chol_solve(d_LT32, d_LN32, d_DI32, m, d_pan_off, d_pan_row, d_x32, g.max_npan, st, d_bs));
        k_s_residual<<<nsm_blocks, TB, 0, st>>>(d_S, d_x32, d_bs, m, d_tfirst, d_tlast, d_y32);
        chk(chol_solve(d_LT32, d_LN32, d_DI32, m, d_pan_off, d_pan_row, d_y32, g.max_npan, st, nullptr, d_x32, d_bs));
        chk(cudaGetLastError());
        return true;
    };
    // state c -> tape slot s
    auto save_state = [&](int c, int s) {
        chk(cudaMemcpyAsync(d_tape_c + (size_t)s * nc, cams[c], sizeof(CamState) * nc, cudaMemcpyDeviceToDevice, st));
        chk(cudaMemcpyAsync(d_tape_x + (size_t)s * 4 * np, A.x[c], sizeof(double) * 4 * np, cudaMemcpyDeviceToDevice, st));
    };
    if (vjp && !vjp->replay) vjp->lambdas.clear();
    const bool replay = vjp && vjp->replay;
    const int n_out = replay ? (int)vjp->lambdas.size() : lm.iterations;
    out.trace.assign(n_out + 1, 0.0);
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
    if (replay) {
        // the given steps, each accepted: x <- x [+] (H + lambda_s I)^-1 b at the current state
        for (int s = 0; s < n_out; ++s) {
            const double lam = vjp->lambdas[s];
            save_state(cur, s);
            linearize(cur);
            k_schur_points<Real><<<pblocks, TB, 0, st>>>(A, D, lam, camr[cur], A.x[cur], d_part);
            bool ok = sum_part(pblocks, false) == 0.0;
            if (nfc > 0) {
                assemble_S(lam);
                ok = factor_S() && ok;
                if (ok) chk(chol_solve(d_LT, d_LN, d_DI, m, d_pan_off, d_pan_row, d_bs, g.max_npan, st));
                chk(cudaGetLastError());
            }
            if (e != cudaSuccess) return e;
            if (!ok) {
                out.status = NAV_BA_ERR_UNSUPPORTED;
                vjp->why = "replayed step " + std::to_string(s) + ": the damped system is not positive definite";
                return cudaSuccess;
            }
            k_update_cams<Real><<<cblocks, TB, 0, st>>>(cams[cur], cams[cur ^ 1], camr[cur ^ 1], d_cam_free, nc, d_bs, d_U,
                                                         lam, d_part);
            k_update_points<Real><<<pblocks, TB, 0, st>>>(A, D, lam, d_bs, cur, d_part);
            chk(cudaGetLastError());
            cur ^= 1;
            chi = cost_of(cur, true);
            if (e != cudaSuccess) return e;
            out.trace[s + 1] = chi;
            lambda = lam;
        }
        out.iterations_done = out.accepted = n_out;
    }
    for (int it = 0; !replay && out.termination == NAV_BA_TERM_ITERATIONS && it < lm.iterations; ++it) {
        A.edge_ep = d_ep[cur];  // mixed form: the FP64 cost pass's residuals of this state
        linearize(cur);
        if (nk) {
            k_lin_intr_points<Real><<<pblocks, TB, 0, st>>>(A, D, camr[cur], A.x[cur], d_kp, d_part);
            double v5[5];
            sum_parts(pblocks, 5, v5);
            Kk[0] = v5[0]; Kk[1] = v5[1]; Kk[2] = v5[2];
            gk[0] = v5[3]; gk[1] = v5[4];
            if (nfc > 0) {
                k_lin_intr_cams<Real><<<iblocks, TB, 0, st>>>(A, d_items, n_items, d_list, d_fcam, camr[cur], A.x[cur],
                                                              d_hpart);
                k_reduce_items<<<(nfc * 12 + TB - 1) / TB, TB, 0, st>>>(d_hpart, 12, 12, d_item_off, nfc, d_Hck, 12);
                chk(cudaGetLastError());
            }
        }
        if (e != cudaSuccess) return e;
        // the largest Hessian diagonal entry of this linearization, read back where first needed
        double maxdiag = -1.0;
        auto get_maxdiag = [&]() -> double {
            if (maxdiag < 0.0) {
                double mxp, mxc;
                lin_maxima(mxp, mxc);
                if (nk) mxc = std::max(mxc, std::max(std::fabs(Kk[0]), std::fabs(Kk[2])));
                maxdiag = std::max(mxp, mxc);
            }
            return maxdiag;
        };
        if (it == 0) {
            lambda = lm.initial_lambda > 0 ? lm.initial_lambda : lm.tau * get_maxdiag();
            nu = 2.0;
        }
        int trial_pit = 0;
        bool trial_ok = true;
        double rho = 0.0;
        int q = 0;
        do {
            const double lam_use = (debug_S && it == 0 && q == 0) ? debug_lambda : lambda;
            // point blocks whose V + lambda I is not positive definite: counted into the trial's
            // read-back (the trial is then rejected; the work between is discarded)
            k_schur_points<Real><<<pblocks, TB, 0, st>>>(A, D, lam_use, camr[cur], A.x[cur], d_tpart);
            bool ok = true, okh_deferred = false;
            double dk[2] = {0.0, 0.0};
            if (pcg && mt > 0) {
                if (pcg_i) k_pcg_pack<Real><<<nsm_blocks, TB, 0, st>>>(A, ne, d_list, ncl, d_apm, d_acm);
                // right-hand side and block-Jacobi preconditioner of the reduced system [cameras; k]
                chk(cudaMemcpyAsync(d_ok, hflag + 2, sizeof(int32_t), cudaMemcpyHostToDevice, st));
                if (nfc > 0 && pcg_x) {
                    // S_ab (block rows, both triangles) and b' from the pair lists, then the factors
                    chk(cudaMemsetAsync(d_flags, 0, sizeof(int32_t) * (2 + g.blocks.size()), st));
                    k_schur_blocks<Real><<<std::max(1, std::min(nsm_blocks, (n_sitems * 32 + TB - 1) / TB)), TB, 0, st>>>(
                        A, d_blocks, d_boff, d_sitems, n_sitems, d_pairs, d_U, lam_use, nullptr, 0, d_bs, d_Sb,
                        d_bslot, d_next, d_sdone, d_spart, kPairChunk);
                    k_pcg_precond_blocks<Real><<<(nfc + TB - 1) / TB, TB, 0, st>>>(d_Sb, d_rs_dslot, nfc, d_pc, d_pcinv, d_ok);
                    chk(cudaGetLastError());
                } else if (nfc > 0) {
                    k_pcg_diag_items<Real><<<iblocks, TB, 0, st>>>(A, d_items, n_items, d_list, d_upart);
                    k_reduce_items<<<(nfc * 27 + TB - 1) / TB, TB, 0, st>>>(d_upart, 28, 27, d_item_off, nfc, d_aat, 28);
                    k_pcg_precond<<<(nfc + TB - 1) / TB, TB, 0, st>>>(d_U, d_aat, nfc, lam_use, d_pc, d_bs, d_ok);
                    chk(cudaGetLastError());
                }
                double pkh[3] = {1.0, 0.0, 1.0};
                double skk[3] = {0.0, 0.0, 0.0};
                if (nk) {
                    k_schur_intr_points<Real><<<pblocks, TB, 0, st>>>(A, D, d_kp, d_pb, d_part);
                    double v5[5];
                    sum_parts(pblocks, 5, v5);
                    // P_k = H_kk + lambda I - sum B B^T (2x2 Cholesky on the host); b'_k = g_k - sum B t
                    const double p00 = Kk[0] + lam_use - v5[0], p01 = Kk[1] - v5[1], p11 = Kk[2] + lam_use - v5[2];
                    const double l00 = p00 > 0 ? std::sqrt(p00) : 1.0;
                    const double l10 = p01 / l00;
                    const double d11 = p11 - l10 * l10;
                    const double l11 = d11 > 0 ? std::sqrt(d11) : 1.0;
                    if (!(p00 > 0) || !(d11 > 0)) ok = false;
                    pkh[0] = l00; pkh[1] = l10; pkh[2] = l11;
                    skk[0] = p00; skk[1] = p01; skk[2] = p11;
                    if (pcg_x && nfc > 0) {
                        k_pcg_xak_items<Real><<<iblocks, TB, 0, st>>>(A, d_items, n_items, d_list, d_pb, d_hpart);
                        k_reduce_items<<<(nfc * 12 + TB - 1) / TB, TB, 0, st>>>(d_hpart, 12, 12, d_item_off, nfc, d_xak, 12);
                        chk(cudaGetLastError());
                    }
                    const double bk[2] = {gk[0] - v5[3], gk[1] - v5[4]};
                    const double kv[6] = {Kk[0], Kk[1], Kk[2], pkh[0], pkh[1], pkh[2]};
                    chk(cudaMemcpyAsync(d_kvals, kv, sizeof(kv), cudaMemcpyHostToDevice, st));
                    chk(cudaMemcpyAsync(d_bs + m, bk, sizeof(bk), cudaMemcpyHostToDevice, st));
                } else {
                    chk(cudaMemcpyAsync(d_kvals + 3, pkh, sizeof(pkh), cudaMemcpyHostToDevice, st));
                }
                PcgVec v;
                v.x = d_vec;
                v.r = d_vec + mt;
                v.z = d_vec + 2LL * mt;
                v.p = d_vec + 3LL * mt;
                v.q = d_vec + 4LL * mt;
                v.sc = d_vec + 5LL * mt;
                v.pf = d_pf;
                v.npf = 6 * nfc;
                PcgArgs<Real> PA;
                PA.A = A;
                PA.np = np;
                PA.ne = ne;
                PA.ncl = ncl;
                PA.nfc = nfc;
                PA.nk = nk;
                PA.mt = mt;
                PA.apm = d_apm;
                PA.acm = d_acm;
                PA.cm_pt = d_cmpt;
                PA.items = d_items;
                PA.n_items = n_items;
                PA.item_off = d_item_off;
                PA.pt_b = d_pb;
                PA.pt_t2 = d_t2;
                PA.camp = d_camp;
                PA.U = d_U;
                PA.Hck = d_Hck;
                PA.kk = d_kvals;
                PA.pc = d_pc;
                PA.b = d_bs;
                PA.lambda = lam_use;
                PA.v = v;
                PA.part = d_ppart;
                PA.max_it = lm.pcg_max_iterations;
                PA.tol2 = lm.pcg_tolerance * lm.pcg_tolerance;
                PA.iters = d_pit;
                PA.phase = d_phase;
                if (pcg_x) {
                    PcgXArgs<Real> XA;
                    XA.Sb = d_Sb;
                    XA.rs_off = d_rs_off;
                    XA.rs_col = d_rs_col;
                    XA.Hck = d_Hck;
                    XA.Xak = d_xak;
                    XA.pcinv = d_pcinv;
                    XA.kk = d_kvals;
                    for (int i = 0; i < 3; ++i) XA.skk[i] = skk[i];
                    XA.b = d_bs;
                    XA.x = v.x;
                    XA.r = v.r;
                    XA.z = v.z;
                    XA.q = v.q;
                    XA.p[0] = v.p;
                    XA.p[1] = d_vec + 5LL * mt;
                    XA.zr = d_zpr;
                    XA.pr[0] = d_zpr + 8LL * std::max(1, nfc);
                    XA.pr[1] = d_zpr + 16LL * std::max(1, nfc);
                    XA.part = d_ppart;
                    XA.nfc = nfc;
                    XA.nk = nk;
                    XA.max_it = lm.pcg_max_iterations;
                    XA.tol2 = PA.tol2;
                    XA.iters = d_pit;
                    XA.phase = d_phase;
                    void* kargs[] = {&XA};
                    chk(cudaLaunchCooperativeKernel((const void*)k_pcg_explicit<Real>, dim3(pcg_grid), dim3(256), kargs, 0,
                                                    st));
                } else {
                    void* kargs[] = {&PA};
                    chk(cudaLaunchCooperativeKernel((const void*)k_pcg_solve<Real>, dim3(pcg_grid), dim3(256), kargs, 0, st));
                }
                chk(cudaMemcpyAsync(hflag + 1, d_pit, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
                chk(cudaMemcpyAsync(d_bs, v.x, sizeof(double) * mt, cudaMemcpyDeviceToDevice, st));
                chk(cudaMemcpyAsync(hflag, d_ok, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
                if (nk) chk(cudaMemcpyAsync(hdk, v.x + m, sizeof(dk), cudaMemcpyDeviceToHost, st));
                chk(cudaStreamSynchronize(st));
                if (e != cudaSuccess) return e;
                const int32_t pit = hflag[1], okh = hflag[0];
                if (nk) {
                    dk[0] = hdk[0];
                    dk[1] = hdk[1];
                }
                pcg_total += pit;
                trial_pit = pit;
                ok = ok && okh != 0;
                if (!ok) {
                    chk(cudaMemsetAsync(d_bs, 0, sizeof(double) * mt, st));
                    dk[0] = dk[1] = 0.0;
                }
                if (nk) k_fold_intr<Real><<<pblocks, TB, 0, st>>>(A, D, d_pb, dk[0], dk[1]);
            } else if (nfc > 0) {
                assemble_S(lam_use);
                if (debug_S) {
                    debug_S->assign((size_t)m * m + m, 0.0);
                    chk(cudaMemcpyAsync(debug_S->data(), d_S, sizeof(double) * m * m, cudaMemcpyDeviceToHost, st));
                    chk(cudaMemcpyAsync(debug_S->data() + (size_t)m * m, d_bs, sizeof(double) * m, cudaMemcpyDeviceToHost, st));
                    chk(cudaStreamSynchronize(st));
                    return e;
                }
                if (mixed_chol) {
                    ok = solve_S_mixed(lam_use, get_maxdiag(), okh_deferred) && ok;
                } else {
                    // a failed factorization rejects the trial: its flag is read with the trial's sums
                    ok = factor_S(true) && ok;
                    okh_deferred = true;
                    if (ok) chk(chol_solve(d_LT, d_LN, d_DI, m, d_pan_off, d_pan_row, d_bs, g.max_npan, st));
                }
                if (e != cudaSuccess) return e;
                if (!ok) chk(cudaMemsetAsync(d_bs, 0, sizeof(double) * m, st));
                chk(cudaGetLastError());
            }
            k_update_trial<Real><<<ucblocks + pblocks, TB, 0, st>>>(
                A, D, lambda, d_bs, cur, ucblocks, pblocks, d_tpart + pblocks + ucblocks, cams[cur], cams[cur ^ 1],
                camr[cur ^ 1], d_cam_free, nc, d_U, d_tpart + pblocks, mixed ? d_camd : nullptr);
            set_radial(A.intr, kcur[0] + dk[0], kcur[1] + dk[1]);
            {  // the trial cost (FP64 in both forms; the mixed form's FP64 cameras from the update)
                const int buf = cur ^ 1;
                double* cpart = d_tpart + 2LL * pblocks + ucblocks;
                if (mixed) {
                    k_cost<double, Real><<<pblocks, TB, 0, st>>>(A, D, d_camd, A.x[buf], cpart, d_ep[buf]);
                } else {
                    k_cost<Real, Real><<<pblocks, TB, 0, st>>>(A, D, camr[buf], A.x[buf], cpart);
                }
                chk(cudaGetLastError());
            }
            // the trial's one read-back
            const double* tp = hpart_trial;
            chk(cudaMemcpyAsync(hpart_trial, d_tpart, sizeof(double) * ntp, cudaMemcpyDeviceToHost, st));
            if (okh_deferred) chk(cudaMemcpyAsync(hflag, d_fail, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
            chk(cudaStreamSynchronize(st));
            if (e != cudaSuccess) return e;
            const int32_t okd = okh_deferred ? (hflag[0] == 0) : 1;
            double npd = 0.0, scale_c = 0.0, scale_p = 0.0, chi_new = 0.0;
            for (int k = 0; k < pblocks; ++k) npd += tp[k];
            for (int k = 0; k < ucblocks; ++k) scale_c += tp[pblocks + k];
            for (int k = 0; k < pblocks; ++k) scale_p += tp[pblocks + ucblocks + k];
            for (int k = 0; k < pblocks; ++k) chi_new += tp[2 * pblocks + ucblocks + k];
            double scale = scale_c + scale_p;
            scale += dk[0] * (lambda * dk[0] + gk[0]) + dk[1] * (lambda * dk[1] + gk[1]);
            if (npd != 0.0 || okd == 0) ok = false;
            if (!ok) chi_new = DBL_MAX;
            trial_ok = ok;
            rho = chi - chi_new;
            scale += 1e-3;
            rho /= scale;
            // a failed damped system is a rejected trial (as g2o's DBL_MAX trial cost makes it), also
            // when the failed point blocks left the step scale non-finite
            if (!ok) rho = -DBL_MAX;
            if (trial_log)
                fprintf(stderr, "[navba grid] it %d trial %d lambda %.3e (%.3e of max diag) ok %d pcg %d cost %.9e rho %.3e\n",
                        it, q, lam_use, lam_use / get_maxdiag(), trial_ok ? 1 : 0, trial_pit, chi_new, rho);
            if (rho > 0 && std::isfinite(chi_new)) {
                if (vjp) {  // tape: the state before this step and its damping
                    save_state(cur, (int)vjp->lambdas.size());
                    vjp->lambdas.push_back(lam_use);
                }
                double alpha = 1.0 - std::pow(2 * rho - 1, 3.0);
                alpha = std::min(alpha, 2.0 / 3.0);
                lambda *= std::max(1.0 / 3.0, alpha);
                nu = 2.0;
                chi = chi_new;
                ++out.accepted;
                cur ^= 1;
                kcur[0] = A.intr.k1;
                kcur[1] = A.intr.k2;
            } else {
                lambda *= nu;
                nu *= 2;
                ++out.rejected;
                set_radial(A.intr, kcur[0], kcur[1]);
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
    out.final_cost = chi;
    out.final_lambda = lambda;
    out.k1 = kcur[0];
    out.k2 = kcur[1];
    out.pcg_iterations = pcg_total;
    k_depth_count<Real><<<pblocks, TB, 0, st>>>(A, D, cams[cur], A.x[cur], d_part);
    chk(cudaGetLastError());
    out.depth_nonpos = (int32_t)sum_part(pblocks, false);
    out.trace.resize(out.iterations_done + 1);
    out.cams.resize(nc);
    out.points.resize(4LL * np);
    chk(cudaMemcpyAsync(out.cams.data(), cams[cur], sizeof(CamState) * nc, cudaMemcpyDeviceToHost, st));
    chk(cudaMemcpyAsync(out.points.data(), A.x[cur], sizeof(double) * 4 * np, cudaMemcpyDeviceToHost, st));
    chk(cudaStreamSynchronize(st));
    if constexpr (std::is_same<Real, double>::value) {
        if (bwd && e == cudaSuccess && out.status == NAV_BA_OK) {
            // ---- backward over the taped steps (vjp_device.cuh) ----
            const int ns = (int)vjp->lambdas.size();
            const int rblocks = (nfc * 6 + TB - 1) / TB;
            // per free camera: sum of the edge vectors (edge adjoints, or A_e t_p with lt) over its items
            auto cam_sum = [&](const double* src, bool lt) {
                k_vjp_cam_items<<<iblocks, TB, 0, st>>>(A, d_items, n_items, d_list, src, lt, d_ipart);
                k_reduce_items<<<rblocks, TB, 0, st>>>(d_ipart, 8, 6, d_item_off, nfc, d_ctmp, 6);
                chk(cudaGetLastError());
            };
            double kb[4] = {0, 0, 0, 0};
            auto add_k = [&]() {
                double v4[4];
                sum_parts(pblocks, 4, v4);
                for (int k = 0; k < 4; ++k) kb[k] += v4[k];
            };
            double* xb = d_cb[0];  // left-tangent adjoint of the current step's output cameras
            double* xa = d_cb[1];
            chk(cudaMemsetAsync(d_uvbar, 0, sizeof(double) * 2 * ne, st));
            if (nfc > 0) {
                chk(cudaMemsetAsync(xb, 0, sizeof(double) * 6 * nfc, st));
                k_vjp_seed_cams<<<cblocks, TB, 0, st>>>(cams[cur], d_cam_free, nc, d_posebar, xb);
            }
            k_vjp_seed_points<<<(np + TB - 1) / TB, TB, 0, st>>>(d_ptbar, np, d_pbar);
            // the final cost's term at the final state
            k_vjp_edges<<<pblocks, TB, 0, st>>>(A, np, camr[cur], A.x[cur], nullptr, nullptr, nullptr, nullptr,
                                                vjp->cost_bar, d_pbar, d_eadj, d_uvbar, d_part);
            chk(cudaGetLastError());
            add_k();
            if (nfc > 0) {
                cam_sum(d_eadj, false);
                k_vjp_axpy<<<rblocks, TB, 0, st>>>(xb, d_ctmp, 1.0, 6 * nfc);
            }
            for (int s = ns - 1; s >= 0 && e == cudaSuccess; --s) {
                const double lam = vjp->lambdas[s];
                // the state before step s, its linearization and factorization (recomputed)
                chk(cudaMemcpyAsync(cams[0], d_tape_c + (size_t)s * nc, sizeof(CamState) * nc, cudaMemcpyDeviceToDevice, st));
                chk(cudaMemcpyAsync(A.x[0], d_tape_x + (size_t)s * 4 * np, sizeof(double) * 4 * np,
                                    cudaMemcpyDeviceToDevice, st));
                k_cams_real<double><<<cblocks, TB, 0, st>>>(cams[0], nc, camr[0]);
                linearize(0);
                k_schur_points<double><<<pblocks, TB, 0, st>>>(A, D, lam, camr[0], A.x[0], d_part);
                bool ok = sum_part(pblocks, false) == 0.0;
                if (nfc > 0) {
                    assemble_S(lam);
                    ok = factor_S() && ok;
                }
                if (e != cudaSuccess) break;
                if (!ok) {
                    out.status = NAV_BA_ERR_UNSUPPORTED;
                    vjp->why = "backward step " + std::to_string(s) + ": the damped system is not positive definite";
                    return cudaSuccess;
                }
                // the step: dx_c (in d_bs), dx_p
                if (nfc > 0) chk(chol_solve(d_LT, d_LN, d_DI, m, d_pan_off, d_pan_row, d_bs, g.max_npan, st));
                k_vjp_point_solve<<<pblocks, TB, 0, st>>>(A, np, d_lt, 12, 6, d_bs, d_dp);
                // adjoint through [+]: rc = J_l^T xbar'_c, xa = Ad^T xbar'_c; r_p = xbar'_p
                if (nfc > 0) k_vjp_cams_step<<<(nfc + 127) / 128, 128, 0, st>>>(d_bs, xb, d_rc, xa, nfc);
                // adjoint solve u = (H + lambda I)^-1 r with the same factorization
                k_vjp_lt_points<<<pblocks, TB, 0, st>>>(A, np, d_pbar, d_tr);
                if (nfc > 0) {
                    cam_sum(d_tr, true);
                    chk(cudaMemcpyAsync(d_uc, d_rc, sizeof(double) * m, cudaMemcpyDeviceToDevice, st));
                    k_vjp_axpy<<<rblocks, TB, 0, st>>>(d_uc, d_ctmp, -1.0, m);
                    chk(chol_solve(d_LT, d_LN, d_DI, m, d_pan_off, d_pan_row, d_uc, g.max_npan, st));
                }
                k_vjp_point_solve<<<pblocks, TB, 0, st>>>(A, np, d_tr, 4, 0, d_uc, d_up);
                // grad psi at the state: points into d_pbar, cameras into xa, observations, intrinsics
                k_vjp_edges<<<pblocks, TB, 0, st>>>(A, np, camr[0], A.x[0], nfc > 0 ? d_uc : nullptr, d_up,
                                                    nfc > 0 ? d_bs : nullptr, d_dp, 0.0, d_pbar, d_eadj, d_uvbar, d_part);
                chk(cudaGetLastError());
                add_k();
                if (nfc > 0) {
                    cam_sum(d_eadj, false);
                    k_vjp_axpy<<<rblocks, TB, 0, st>>>(xa, d_ctmp, 1.0, 6 * nfc);
                }
                std::swap(xa, xb);
            }
            if (e != cudaSuccess) return e;
            vjp->uv_bar.assign(2LL * ne, 0.0);
            std::vector<double> pb(4LL * np), cb(6LL * nfc1, 0.0);
            chk(cudaMemcpyAsync(vjp->uv_bar.data(), d_uvbar, sizeof(double) * 2 * ne, cudaMemcpyDeviceToHost, st));
            chk(cudaMemcpyAsync(pb.data(), d_pbar, sizeof(double) * 4 * np, cudaMemcpyDeviceToHost, st));
            if (nfc > 0) chk(cudaMemcpyAsync(cb.data(), xb, sizeof(double) * 6 * nfc, cudaMemcpyDeviceToHost, st));
            chk(cudaStreamSynchronize(st));
            if (e != cudaSuccess) return e;
            for (int k = 0; k < 4; ++k) vjp->intr_bar[k] = kb[k];
            vjp->pt_bar.assign(3LL * np, 0.0);
            for (int p = 0; p < np; ++p)
                if (h.pt_free[p] >= 0)
                    for (int j = 0; j < 3; ++j) vjp->pt_bar[3LL * p + j] = pb[4LL * p + j];
            vjp->cam_bar.assign(6LL * nc, 0.0);
            for (int c = 0; c < nc; ++c)
                if (h.cam_free[c] >= 0)
                    for (int j = 0; j < 6; ++j) vjp->cam_bar[6LL * c + j] = cb[6LL * h.cam_free[c] + j];
        }
    }
    return e;
}

}  // namespace

cudaError_t grid_solve(const HostWindow& h, const LmOptions& lm, const Intr& intr, int precision, cudaStream_t stream,
                       HostPool* pool, GridWorkspace* ws, GridResult& out, double debug_lambda,
                       std::vector<double>* debug_S, GridVjp* vjp) {
    if (precision == NAV_BA_MIXED)
        return grid_solve_typed<float>(h, lm, intr, stream, pool, ws, out, debug_lambda, debug_S,
                                       vjp && !vjp->backward ? vjp : nullptr);
    return grid_solve_typed<double>(h, lm, intr, stream, pool, ws, out, debug_lambda, debug_S, vjp);
}

}  // namespace navba
