// window_engine.cu - batched bundle adjustment: one persistent kernel solves many windows.
//
// A thread-block cluster of C CTAs (C = 1, 2, 4 or 8, picked by the autotuner) solves one
// window at a time: rank 0 takes the next window from a work queue (ordered by the host,
// largest first) and the cluster runs that window's whole Levenberg-Marquardt loop before taking
// the next, so a batch of uneven windows is one launch.  Every CTA keeps its own copy of the
// window's camera states; rank 0 keeps the camera blocks of H and the reduced camera system S
// (packed lower triangle, FP64) in its shared memory, the other ranks write into it through
// distributed shared memory.  Per-point and per-edge quantities live in global memory; with C
// CTAs per window only 1/C as many windows are in flight, which keeps their scratch in L2.
//
// One LM iteration (g2o OptimizationAlgorithmLevenberg::solve semantics as used by nav24's
// GraphOptim::solve, core/backEnd/BE_GraphOptim.cpp:67-68):
//   linearize  point-major, thread per point: residual, pose/point Jacobians and Huber weight per
//              edge (EdgeSE3ProjectXYZ::computeError/linearizeOplus, OptimizableTypes.hpp:102-107,
//              OptimizableTypes.cpp:140-161); V_p, g_p; the FP64 form stores W_e = w Jc^T Jp.
//              camera-major, warp per camera: the edges are re-linearized and U_c, g_c summed by
//              warp shuffles (nothing per edge is stored for them).
//   trial      point-major: V_p + lambda I = R R^T (3x3 Cholesky), L = R^-1, A_e = W_e L^T (the
//              mixed form recomputes W_e from the edge's Jacobians), t_p = L g_p, so that
//              W V^-1 W^T = A A^T and W V^-1 g = A t.
//              warp per 6x6 block of S over the block's pair list (built once per window,
//              deterministic order): S_ab = [a==b](U_a + lambda I) - sum A_i A_j^T, summed in
//              registers and reduced by shuffles, no atomics; b'_a = g_a - sum A_i t_p.
//              FP64 Cholesky of S (rank 0); dx_p = L^T (t_p - sum A_i^T dx_c); T <- exp(dx) T;
//              cost of the trial state (mixed form: FP32 residual changes, fused with the point
//              update); gain ratio, accept/reject and damping update.
// Real is double (plain FP64 form) or float (mixed form: residuals, Jacobians, H blocks and the
// Schur products in FP32; S, its Cholesky, the states, the SE(3) update and cost sums in FP64).
#include <algorithm>
#include <cfloat>
#include <cstdio>
#include <cstdlib>
#include <thread>

#include <cooperative_groups.h>

#include "engine.hpp"
#include "lm_device.cuh"

namespace cg = cooperative_groups;

namespace navba {
namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kMaxCluster = 8;
constexpr int kMaxBlocks = kWinMaxFreeCams * (kWinMaxFreeCams + 1) / 2;

struct SmemHead {
    double U[kWinMaxFreeCams][28];         // rank 0: packed lower U (21) | g_c (6) | pad
    double cred[2][kMaxCluster][4];        // rank 0: cluster reduction slots (double-buffered)
    double red[2 * 16 * 3];                // per CTA: block reduction scratch
    double bcast[4];                       // per CTA: reduced values
    int32_t fcam[kWinMaxFreeCams];         // per CTA: free index -> local camera
    int32_t loff[kWinMaxCams + 1];         // per CTA: camera-major list offsets
    int32_t lcnt[kWinMaxCams];             // per CTA: edges per camera (free cameras)
    int32_t poff[kMaxBlocks + 1];          // rank 0: pair-list offsets of the S blocks
    int32_t pcnt[kMaxBlocks];              // rank 0: pairs per S block
    int32_t whist[16][kWinMaxFreeCams];    // per warp: pair counts / cursors of one block row
    int32_t cur, ok, win, slot;
    int32_t next_blk;  // a CTA solving a window alone: the Schur-block work counter
    double lm[4];    // the LM decision of a trial: rho, lambda, nu, chi (made by thread 0)
    int32_t lm_acc;  // the trial was accepted
};

// Offsets of the dynamic part of shared memory (after SmemHead), shared by host and device.
struct Dyn {
    size_t cams, camr, camd, camdel, dcl, dclr, S, bs, rinv, s32, v32, total;
};

NAVBA_HD size_t align16(size_t x) { return (x + 15) & ~(size_t)15; }

NAVBA_HD Dyn dyn_layout(int max_m, int max_ncam, int real_size) {
    Dyn d;
    size_t o = align16(sizeof(SmemHead));
    d.cams = o; o = align16(o + sizeof(CamState) * 2 * max_ncam);
    d.camr = o; o = align16(o + (size_t)real_size * 2 * max_ncam * 12);
    d.camd = o; o = align16(o + sizeof(double) * 2 * max_ncam * 12);
    d.camdel = o; o = align16(o + (size_t)real_size * max_ncam * 12);
    d.dcl = o;  o = align16(o + sizeof(double) * max_m);
    d.dclr = o; o = align16(o + (size_t)real_size * max_m);
    // S (FP64 form; the mixed form keeps its FP64 S in global memory, WinArgs::s_glob), at least
    // the camera-list counting sort's [16][kWinMaxCams] table, which borrows it
    const size_t s_bytes = real_size == 4 ? 0 : sizeof(double) * ((size_t)max_m * (max_m + 1) / 2);
    d.S = o;    o = align16(o + std::max(s_bytes, sizeof(int32_t) * 16 * (size_t)kWinMaxCams));
    d.bs = o;   o = align16(o + sizeof(double) * max_m);
    d.rinv = o; o = align16(o + sizeof(double) * max_m);
    // mixed form: the FP32 factor of S and three FP32 vectors (1/L_jj, solution, correction)
    const bool f32 = real_size == 4;
    d.s32 = o;  o = align16(o + (f32 ? sizeof(float) * ((size_t)max_m * (max_m + 1) / 2) : 0));
    d.v32 = o;  o = align16(o + (f32 ? sizeof(float) * 3 * max_m : 0));
    d.total = o;
    return d;
}

// Barrier over the CTAs solving the current window: the whole cluster, or the CTA alone when it
// solves a window by itself (the single-CTA phase of a clustered launch).
__device__ __forceinline__ void csync(const CC& c) {
    if (c.csize > 1) cg::this_cluster().sync();
    else __syncthreads();
}

// Decode lower-triangle block index blk = a (a + 1) / 2 + b, b <= a.
__device__ __forceinline__ void decode_block(int blk, int& a, int& b) {
    a = (int)((sqrtf(8.0f * (float)blk + 1.0f) - 1.0f) * 0.5f);
    while ((a + 1) * (a + 2) / 2 <= blk) ++a;
    while (a * (a + 1) / 2 > blk) --a;
    b = blk - a * (a + 1) / 2;
}

// The S blocks a warp takes: in a cluster, a fixed share (warp gw takes blocks gw, gw + CW, ...);
// in a CTA solving its window alone, the next one from a shared-memory counter, diagonal blocks
// first (each carries every observation of its camera, the longest pair lists), so that no warp
// is left with several of them while the others wait at the barrier.  next() returns false when
// the blocks are exhausted; a, b, blk are the block's camera pair and packed index.
struct BlockSchedule {
    int k, nblk, nfc;
    bool dynamic;
    __device__ BlockSchedule(const CC& c, int nfc_) : nblk(nfc_ * (nfc_ + 1) / 2), nfc(nfc_), dynamic(c.csize == 1) {
        k = dynamic ? -1 : c.gw - c.CW;
    }
    __device__ bool next(const CC& c, int& a, int& b, int& blk) {
        if (dynamic) {
            int j = 0;
            if (c.lane == 0) j = atomicAdd(&c.s->next_blk, 1);
            k = __shfl_sync(0xffffffffu, j, 0);
            if (k >= nblk) return false;
            if (k < nfc) {
                a = b = k;
            } else {  // off-diagonal o = a (a - 1) / 2 + b, b < a
                const int o = k - nfc;
                a = (int)((1.0f + sqrtf(8.0f * (float)o + 1.0f)) * 0.5f);
                while (a * (a - 1) / 2 > o) --a;
                while ((a + 1) * a / 2 <= o) ++a;
                b = o - a * (a - 1) / 2;
            }
            blk = a * (a + 1) / 2 + b;
            return true;
        }
        k += c.CW;
        if (k >= nblk) return false;
        blk = k;
        decode_block(blk, a, b);
        return true;
    }
};

// Sums (or a max for the first value when MAX0) of three per-thread values over the whole
// cluster; every thread of every CTA gets the same result (fixed reduction order).
template <bool MAX0>
__device__ double3 cluster_reduce3(CC& c, double a, double b, double d) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const double ta = __shfl_down_sync(kFull, a, o);
        a = MAX0 ? fmax(a, ta) : a + ta;
        b += __shfl_down_sync(kFull, b, o);
        d += __shfl_down_sync(kFull, d, o);
    }
    SmemHead& s = *c.s;
    __syncthreads();
    if (c.lane == 0) {
        s.red[3 * c.wid] = a;
        s.red[3 * c.wid + 1] = b;
        s.red[3 * c.wid + 2] = d;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double ra = s.red[0], rb = s.red[1], rd = s.red[2];
        for (int i = 1; i < c.nw; ++i) {
            ra = MAX0 ? fmax(ra, s.red[3 * i]) : ra + s.red[3 * i];
            rb += s.red[3 * i + 1];
            rd += s.red[3 * i + 2];
        }
        double* slot = c.s0->cred[s.slot][c.rank];
        slot[0] = ra;
        slot[1] = rb;
        slot[2] = rd;
    }
    csync(c);
    if (threadIdx.x == 0) {
        double ra = c.s0->cred[s.slot][0][0], rb = c.s0->cred[s.slot][0][1], rd = c.s0->cred[s.slot][0][2];
        for (int r = 1; r < c.csize; ++r) {
            const double* slot = c.s0->cred[s.slot][r];
            ra = MAX0 ? fmax(ra, slot[0]) : ra + slot[0];
            rb += slot[1];
            rd += slot[2];
        }
        s.bcast[0] = ra;
        s.bcast[1] = rb;
        s.bcast[2] = rd;
        s.slot ^= 1;
    }
    __syncthreads();
    return make_double3(s.bcast[0], s.bcast[1], s.bcast[2]);
}

// Camera-major edge lists of the free cameras and the pair lists of the S blocks.
template <class Real, class Mark>
__device__ void build_lists(const WinArgs<Real>& A, CC& c, const WinDesc& D, int32_t (*wcam)[kWinMaxCams], Mark&& mark) {
    SmemHead& s = *c.s;
    // Camera-major lists of the free cameras' edges, stable (point-major order within a camera): a
    // counting sort by rank 0's warps, each over one contiguous range of the window's edges.  Pass 1
    // counts per (warp, camera) (match + popc), the offsets are camera-major then warp-major, pass 2
    // places each 32-edge chunk's edges of one camera in lane order.
    if (c.rank == 0) {
        const int nw = c.nw;
        for (int k = threadIdx.x; k < nw * kWinMaxCams; k += blockDim.x) wcam[k / kWinMaxCams][k % kWinMaxCams] = 0;
        __syncthreads();
        const int per = (D.ne + nw - 1) / nw;
        const int lo = c.wid * per, hi = min(D.ne, lo + per);
        const unsigned below = (1u << c.lane) - 1u;
        auto cam_of = [&](int e) { return e < hi && A.edge_fc[D.e0 + e] >= 0 ? A.edge_cam[D.e0 + e] : -1; };
        for (int base = lo; base < hi; base += 32) {
            const int cam = cam_of(base + c.lane);
            const unsigned grp = __match_any_sync(kFull, cam);
            if (cam >= 0 && (grp & below) == 0) wcam[c.wid][cam] += __popc(grp);
            __syncwarp();
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            int acc = 0;
            for (int cam = 0; cam < D.ncam; ++cam) {
                s.loff[cam] = acc;
                for (int w = 0; w < nw; ++w) {
                    const int t = wcam[w][cam];
                    wcam[w][cam] = acc;
                    acc += t;
                }
                s.lcnt[cam] = acc - s.loff[cam];
                const int a = A.cam_free[D.cam0 + cam];
                if (a >= 0) s.fcam[a] = cam;
            }
            s.loff[D.ncam] = acc;
        }
        __syncthreads();
        for (int base = lo; base < hi; base += 32) {
            const int e = base + c.lane;
            const int cam = cam_of(e);
            const unsigned grp = __match_any_sync(kFull, cam);
            if (cam >= 0) A.cam_list[D.e0 + wcam[c.wid][cam] + __popc(grp & below)] = D.e0 + e;
            __syncwarp();
            if (cam >= 0 && (grp & below) == 0) wcam[c.wid][cam] += __popc(grp);
            __syncwarp();
        }
    }
    csync(c);  // the lists are in global memory and their offsets in rank 0's head
    if (c.rank != 0) {  // the other CTAs of the cluster take rank 0's offsets
        for (int k = threadIdx.x; k <= D.ncam; k += blockDim.x) s.loff[k] = c.s0->loff[k];
        for (int k = threadIdx.x; k < D.ncam; k += blockDim.x) s.lcnt[k] = c.s0->lcnt[k];
        for (int k = threadIdx.x; k < D.nfc; k += blockDim.x) s.fcam[k] = c.s0->fcam[k];
    }
    __syncthreads();
    mark(14);
    // Schur pairs by block row: the warp of free camera a walks a's edges i and, for each, the other
    // edges j of i's free point whose free camera b <= a; pair (i, j) belongs to block (a, b).
    const int nblk = D.nfc * (D.nfc + 1) / 2;
    int* hist = c.s->whist[c.wid];
    for (int a = c.gw; a < D.nfc; a += c.CW) {
        for (int b = c.lane; b <= a; b += 32) hist[b] = 0;
        __syncwarp();
        const int ca = s.fcam[a];
        const int* list = A.cam_list + D.e0 + s.loff[ca];
        const int cnt = s.lcnt[ca];
        // the list entry's edge is loaded a round ahead; the point's edges' free cameras four at a time
        int ei_n = c.lane < cnt ? list[c.lane] : 0;
        for (int i = c.lane; i < cnt; i += 32) {
            const int gp = D.pt0 + A.edge_pt[ei_n];
            if (i + 32 < cnt) ei_n = list[i + 32];
            if (A.pt_free[gp] < 0) continue;
            const int e0 = A.pt_eoff[gp], e1 = A.pt_eoff[gp + 1];
            for (int ej = e0; ej < e1; ej += 4) {
                int bb[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) bb[u] = ej + u < e1 ? A.edge_fc[ej + u] : -1;
#pragma unroll
                for (int u = 0; u < 4; ++u)
                    if (bb[u] >= 0 && bb[u] <= a) atomicAdd(&hist[bb[u]], 1);  // integer counts: order-independent
            }
        }
        __syncwarp();
        for (int b = c.lane; b <= a; b += 32) c.s0->pcnt[a * (a + 1) / 2 + b] = hist[b];
        __syncwarp();
    }
    csync(c);
    mark(15);
    if (c.rank == 0 && threadIdx.x == 0) {
        int acc = 0;
        for (int k = 0; k < nblk; ++k) {
            s.poff[k] = acc;
            acc += s.pcnt[k];
        }
        s.poff[nblk] = acc;
    }
    csync(c);
    // fill: lanes take 32 consecutive edges of a's list; in warp-uniform rounds every lane emits its
    // next pair; lanes of one round with the same block are placed in lane order (match + rank) and
    // the block's cursor advances, so each block's list is in (list position, point-edge) order
    const int64_t end = D.pair0 + D.npair;
    for (int a = c.gw; a < D.nfc; a += c.CW) {
        for (int b = c.lane; b <= a; b += 32) hist[b] = c.s0->poff[a * (a + 1) / 2 + b];
        __syncwarp();
        const int ca = s.fcam[a];
        const int* list = A.cam_list + D.e0 + s.loff[ca];
        const int cnt = s.lcnt[ca];
        for (int base = 0; base < cnt; base += 32) {
            const int i = base + c.lane;
            int ei = -1, ej = 0, e1 = 0;
            if (i < cnt) {
                ei = list[i];
                const int gp = D.pt0 + A.edge_pt[ei];
                if (A.pt_free[gp] >= 0) {
                    ej = A.pt_eoff[gp];
                    e1 = A.pt_eoff[gp + 1];
                }
            }
            for (;;) {
                int b = -1;
                for (; ej < e1; ++ej) {
                    const int bb = A.edge_fc[ej];
                    if (bb >= 0 && bb <= a) {
                        b = bb;
                        break;
                    }
                }
                if (__ballot_sync(kFull, b >= 0) == 0u) break;
                const unsigned grp = __match_any_sync(kFull, b);
                if (b >= 0) {
                    const int64_t q = D.pair0 + hist[b] + __popc(grp & ((1u << c.lane) - 1u));
                    if (q < end) A.pairs[q] = ((uint32_t)(ei - D.e0) << 16) | (uint32_t)(ej - D.e0);
                }
                __syncwarp();
                if (b >= 0 && (grp >> c.lane) == 1u) hist[b] += __popc(grp);  // the group's highest lane
                __syncwarp();
                if (b >= 0) ++ej;
            }
        }
    }
    csync(c);
}

// Camera-major linearization: U_c, g_c (warp per free camera) into rank 0; returns max |diag U|.
template <class Real>
__device__ double linearize_cameras(const WinArgs<Real>& A, const CC& c, const WinDesc& D, const Real* camr,
                                    const double* X, const Real* XR) {
    const Real delta = (Real)A.lm.huber_delta;
    const SmemHead& s = *c.s;
    double mx = 0.0;
    for (int a = c.gw; a < D.nfc; a += c.CW) {
        const int cam = s.fcam[a];
        const int* list = A.cam_list + D.e0 + s.loff[cam];
        const int cnt = s.lcnt[cam];
        Real cr[12];
        cam_load(camr + 12 * cam, cr);
        Real u[27];
#pragma unroll
        for (int k = 0; k < 27; ++k) u[k] = Real(0);
        // the list position's edge is loaded two rounds ahead and its point one round ahead, so a
        // round waits for one memory latency instead of three dependent ones
        int e_n = c.lane < cnt ? list[c.lane] : 0;
        int gp_n = c.lane < cnt ? D.pt0 + A.edge_pt[e_n] : 0;
        int e_nn = c.lane + 32 < cnt ? list[c.lane + 32] : 0;
        for (int i = c.lane; i < cnt; i += 32) {
            const int e = e_n, gp = gp_n;
            Real Xr[3], z[2];
            point_real(X, XR, gp, Xr);
            obs_real(A, e, z);
            e_n = e_nn;
            if (i + 32 < cnt) gp_n = D.pt0 + A.edge_pt[e_n];
            if (i + 64 < cnt) e_nn = list[i + 64];
            EdgeLin<Real> L;
            edge_linearize<Real>(A.intr, cr, cr + 9, Xr, z, A.lm.robust != 0, delta, L);
            const Real w = L.w;
#pragma unroll
            for (int r = 0; r < 6; ++r)
#pragma unroll
                for (int q = 0; q <= r; ++q) u[tri(r, q)] += w * (L.jc[r] * L.jc[q] + L.jc[6 + r] * L.jc[6 + q]);
            const Real we0 = -w * L.e[0], we1 = -w * L.e[1];
#pragma unroll
            for (int r = 0; r < 6; ++r) u[21 + r] += L.jc[r] * we0 + L.jc[6 + r] * we1;
        }
#pragma unroll
        for (int k = 0; k < 27; ++k)
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) u[k] += __shfl_xor_sync(kFull, u[k], o);
        // lane k widens value k: one FP64 conversion per warp, not one per value
        const Real uk = lane_value<27>(u, c.lane);
        if (c.lane < 27) c.s0->U[a][c.lane] = (double)uk;
        Real dm = Real(0);
#pragma unroll
        for (int r = 0; r < 6; ++r) dm = fmax(dm, fabs(u[tri(r, r)]));
        mx = fmax(mx, (double)dm);
    }
    return mx;
}

// Sums one S block's lane partials over the warp and writes -sum (plus U_a + lambda I on the
// diagonal) into the packed S, and b'_a = g'_a - sum A t on the diagonal.  The reduce-scatter leaves
// each lane the two entries it writes, so each FP64 operation is one warp instruction with all lanes
// active (GB300's FP64 pipe costs 16 cycles per warp instruction, however few lanes are active).
template <class Real>
__device__ __forceinline__ void write_block(const CC& c, int a, int b, Real* acc, Real* accb, double lambda) {
    Real sums[2];
    reduce_scatter36(acc, c.lane, sums[0], sums[1]);
    const int k0 = rs36_slot(c.lane);
    if (a == b) {
#pragma unroll
        for (int k = 0; k < 6; ++k)
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) accb[k] += __shfl_xor_sync(kFull, accb[k], o);
    }
#pragma unroll
    for (int rnd = 0; rnd < 2; ++rnd) {
        const int k = k0 + rnd;
        const int r = k / 6, q = k % 6;
        if (k < 36 && !(a == b && q > r)) {
            double v = -(double)sums[rnd];
            if (a == b) {
                v += c.s0->U[a][tri(r, q)];
                if (r == q) v += lambda;
            }
            c.S0[tri(6 * a + r, 6 * b + q)] = v;
            if (c.S0f) c.S0f[tri(6 * a + r, 6 * b + q)] = (float)v;
        }
    }
    if (a == b) {
        const Real bk = lane_value<6>(accb, c.lane);
        if (c.lane < 6) c.bs0[6 * a + c.lane] = c.s0->U[a][21 + c.lane] - (double)bk;
    }
}

// S blocks from Jacobian-factored records (mixed form, pinhole): per pair (i, j) of block (a, b),
// A_i A_j^T = J_ci^T M J_cj with M = B_i B_j^T (2x2), the J_c rebuilt from each record's (u, v, iz).
__device__ void schur_blocks_jf(const WinArgs<float>& A, const CC& c, const WinDesc& D, double lambda) {
    const float fx = (float)A.intr.fx, fy = (float)A.intr.fy;
    BlockSchedule sched(c, D.nfc);
    int a, b, blk;
    while (sched.next(c, a, b, blk)) {
        const int64_t base = D.pair0 + c.s0->poff[blk];
        const int n = c.s0->pcnt[blk];
        float acc[36], accb[6];
#pragma unroll
        for (int k = 0; k < 36; ++k) acc[k] = 0.f;
#pragma unroll
        for (int k = 0; k < 6; ++k) accb[k] = 0.f;
        uint32_t pr_next = c.lane < n ? A.pairs[base + c.lane] : 0u;
        for (int k = c.lane; k < n; k += 32) {
            const uint32_t pr = pr_next;
            pr_next = k + 32 < n ? A.pairs[base + k + 32] : 0u;  // prefetch the next pair index
            const int ei = D.e0 + (int)(pr >> 16), ej = D.e0 + (int)(pr & 0xffffu);
            float ri[12], rj[12];
            JRec::load(A.edge_a + (long long)JRec::kEdge * ei, ri);
            JRec::load(A.edge_a + (long long)JRec::kEdge * ej, rj);
            const float m00 = ri[3] * rj[3] + ri[4] * rj[4] + ri[5] * rj[5];
            const float m01 = ri[3] * rj[6] + ri[4] * rj[7] + ri[5] * rj[8];
            const float m10 = ri[6] * rj[3] + ri[7] * rj[4] + ri[8] * rj[5];
            const float m11 = ri[6] * rj[6] + ri[7] * rj[7] + ri[8] * rj[8];
            float jj[12], t0[6], t1[6];
            pinhole_jc(fx, fy, rj[0], rj[1], rj[2], jj);
#pragma unroll
            for (int q = 0; q < 6; ++q) {
                t0[q] = m00 * jj[q] + m01 * jj[6 + q];
                t1[q] = m10 * jj[q] + m11 * jj[6 + q];
            }
            float ji[12];
            pinhole_jc(fx, fy, ri[0], ri[1], ri[2], ji);
#pragma unroll
            for (int r = 0; r < 6; ++r)
#pragma unroll
                for (int q = 0; q < 6; ++q) acc[r * 6 + q] += ji[r] * t0[q] + ji[6 + r] * t1[q];
            if (a == b && ei == ej) {
                const float b0 = ri[3] * ri[9] + ri[4] * ri[10] + ri[5] * ri[11];
                const float b1 = ri[6] * ri[9] + ri[7] * ri[10] + ri[8] * ri[11];
#pragma unroll
                for (int r = 0; r < 6; ++r) accb[r] += ji[r] * b0 + ji[6 + r] * b1;
            }
        }
        write_block<float>(c, a, b, acc, accb, lambda);
    }
}

// S blocks (warp per block over its pair list) into rank 0's packed S, and b'.
template <class Real>
__device__ void schur_blocks(const WinArgs<Real>& A, const CC& c, const WinDesc& D, double lambda) {
    if constexpr (sizeof(Real) == 4) {
        if (A.jfact) {
            schur_blocks_jf(A, c, D, lambda);
            return;
        }
    }
    BlockSchedule sched(c, D.nfc);
    int a, b, blk;
    while (sched.next(c, a, b, blk)) {
        const int64_t base = D.pair0 + c.s0->poff[blk];
        const int n = c.s0->pcnt[blk];
        Real acc[36];
        Real accb[6];
#pragma unroll
        for (int k = 0; k < 36; ++k) acc[k] = Real(0);
#pragma unroll
        for (int k = 0; k < 6; ++k) accb[k] = Real(0);
        uint32_t pr_next = c.lane < n ? A.pairs[base + c.lane] : 0u;
        for (int k = c.lane; k < n; k += 32) {
            const uint32_t pr = pr_next;
            pr_next = k + 32 < n ? A.pairs[base + k + 32] : 0u;  // prefetch the next pair index
            const int ei = D.e0 + (int)(pr >> 16), ej = D.e0 + (int)(pr & 0xffffu);
            Real ai[18], aj[18];
            Rec<Real>::load18(A.edge_a + (long long)Rec<Real>::kEdge * ei, ai);
            Rec<Real>::load18(A.edge_a + (long long)Rec<Real>::kEdge * ej, aj);
#pragma unroll
            for (int r = 0; r < 6; ++r)
#pragma unroll
                for (int q = 0; q < 6; ++q)
                    acc[r * 6 + q] += ai[r * 3 + 0] * aj[q * 3 + 0] + ai[r * 3 + 1] * aj[q * 3 + 1] + ai[r * 3 + 2] * aj[q * 3 + 2];
            if (a == b && ei == ej) {
                const Real* t = A.pt_lt + 12LL * (D.pt0 + A.edge_pt[ei]) + 6;
                const Real t0 = t[0], t1 = t[1], t2 = t[2];
#pragma unroll
                for (int r = 0; r < 6; ++r) accb[r] += ai[r * 3 + 0] * t0 + ai[r * 3 + 1] * t1 + ai[r * 3 + 2] * t2;
            }
        }
        write_block<Real>(c, a, b, acc, accb, lambda);
    }
}

// In-place Cholesky (LL^T) of packed lower S (m x m) in this CTA's shared memory, FP64; rinv
// receives 1/L_jj.  Right-looking: per column j, the column is scaled by 1/L_jj (thread per row),
// then the trailing rows are updated (warp per row).  The next pivot's row is the first row of
// warp 0, whose lane 0 takes the pivot right after updating it, so a column costs two barriers.
// One reciprocal square root per column (FP64 divides and square roots are long instruction
// sequences on GB300's FP64 pipe, so the column is scaled by a product); every FP64 product is
// made by one lane only (the pipe's throughput is counted in lanes).
template <class T>
__device__ bool smem_cholesky(T* S, T* rinv, int m, SmemHead& s) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    auto pivot = [&](int j) {  // L_jj and rinv[j]; a pivot that is not positive and finite fails
        const T d = S[tri(j, j)];
        if (!(d > T(0)) || !isfinite(d)) {
            s.ok = 0;
            S[tri(j, j)] = T(1);
            rinv[j] = T(1);
        } else {
            const T r = rsqrt(d);
            S[tri(j, j)] = d * r;
            rinv[j] = r;
        }
    };
    if (threadIdx.x == 0) {
        s.ok = 1;
        if (m > 0) pivot(0);
    }
    __syncthreads();
    for (int j = 0; j < m; ++j) {
        const T ri = rinv[j];
        for (int i = j + 1 + threadIdx.x; i < m; i += blockDim.x) S[tri(i, j)] *= ri;
        __syncthreads();
        for (int i = j + 1 + wid; i < m; i += nw) {
            const T lij = S[tri(i, j)];
            T* Si = S + tri(i, 0);
            for (int k = j + 1 + lane; k <= i; k += 32) Si[k] -= lij * S[tri(k, j)];
            if (i == j + 1 && lane == 0) pivot(j + 1);  // lane 0 updated S[j+1][j+1] itself
        }
        __syncthreads();
    }
    return s.ok != 0;
}

// Solve L L^T x = b in place, FP64, packed L, rinv = 1/diag(L); column-oriented substitution
// with one barrier per column (the owner of the next row finalizes it).
__device__ void smem_chol_solve(const double* L, const double* rinv, int m, double* x) {
    if (m == 0) return;
    if (threadIdx.x == 0) x[0] *= rinv[0];
    __syncthreads();
    for (int j = 0; j < m - 1; ++j) {
        const double xj = x[j];
        for (int i = j + 1 + threadIdx.x; i < m; i += blockDim.x) {
            double v = x[i] - L[tri(i, j)] * xj;
            if (i == j + 1) v *= rinv[i];
            x[i] = v;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) x[m - 1] *= rinv[m - 1];
    __syncthreads();
    for (int j = m - 1; j > 0; --j) {
        const double xj = x[j];
        const double* Lj = L + tri(j, 0);
        for (int i = threadIdx.x; i < j; i += blockDim.x) {
            double v = x[i] - Lj[i] * xj;
            if (i == j - 1) v *= rinv[i];
            x[i] = v;
        }
        __syncthreads();
    }
}

// FP32 Cholesky (LL^T) of packed lower S (m x m) in shared memory, blocked in panels of kNB columns:
// warp 0 factors the panel's diagonal block (row r in lane r, shuffles) and solves the rows below
// it against that block; then every warp applies the panel's rank-kNB update to the trailing
// matrix.  Two block barriers per panel instead of two per column.  rinv receives 1/L_jj; a pivot
// that is not positive and finite fails the factorization (it is replaced by 1 so the pass ends).
constexpr int kNB = 8;
__device__ bool smem_cholesky_blocked(float* S, float* rinv, int m, SmemHead& s) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if (threadIdx.x == 0) s.ok = 1;
    __syncthreads();
    for (int p0 = 0; p0 < m; p0 += kNB) {
        const int pb = min(kNB, m - p0);
        if (wid == 0) {
            float d[kNB];  // lane r < pb: row p0 + r of the diagonal block, columns 0..r
#pragma unroll
            for (int c2 = 0; c2 < kNB; ++c2) d[c2] = (lane < pb && c2 <= lane) ? S[tri(p0 + lane, p0 + c2)] : 0.f;
            bool bad = false;
#pragma unroll
            for (int cc = 0; cc < kNB; ++cc) {
                if (cc >= pb) break;
                const float dc = __shfl_sync(kFull, d[cc], cc);
                const bool colbad = !(dc > 0.f) || !isfinite(dc);
                const float r = colbad ? 1.f : rsqrtf(dc);
                bad = bad || colbad;
                if (lane == cc) d[cc] = colbad ? 1.f : dc * r;
                else if (lane > cc) d[cc] *= r;
                if (lane == 0) rinv[p0 + cc] = r;
#pragma unroll
                for (int j = cc + 1; j < kNB; ++j) {
                    const float ljc = __shfl_sync(kFull, d[cc], j);
                    if (lane >= j) d[j] -= d[cc] * ljc;
                }
            }
            if (bad && lane == 0) s.ok = 0;
#pragma unroll
            for (int c2 = 0; c2 < kNB; ++c2)
                if (lane < pb && c2 <= lane) S[tri(p0 + lane, p0 + c2)] = d[c2];
            __syncwarp();
            // rows below the block: x_c = (x_c - sum_{c' < c} x_c' L_cc') / L_cc
            for (int i = p0 + pb + lane; i < m; i += 32) {
                float* Si = S + tri(i, p0);
                float x[kNB];
#pragma unroll
                for (int c2 = 0; c2 < kNB; ++c2) x[c2] = c2 < pb ? Si[c2] : 0.f;
#pragma unroll
                for (int cc = 0; cc < kNB; ++cc) {
                    if (cc >= pb) break;
                    const float* Dc = S + tri(p0 + cc, p0);
                    float v = x[cc];
#pragma unroll
                    for (int c2 = 0; c2 < cc; ++c2) v -= x[c2] * Dc[c2];
                    x[cc] = v * rinv[p0 + cc];
                }
#pragma unroll
                for (int c2 = 0; c2 < kNB; ++c2)
                    if (c2 < pb) Si[c2] = x[c2];
            }
        }
        __syncthreads();
        const int t0 = p0 + pb;
        for (int i = t0 + wid; i < m; i += nw) {
            const float* Li = S + tri(i, p0);
            float li[kNB];
#pragma unroll
            for (int c2 = 0; c2 < kNB; ++c2) li[c2] = c2 < pb ? Li[c2] : 0.f;
            float* Si = S + tri(i, 0);
            for (int j = t0 + lane; j <= i; j += 32) {
                const float* Lj = S + tri(j, p0);
                float acc = Si[j];
#pragma unroll
                for (int c2 = 0; c2 < kNB; ++c2)
                    if (c2 < pb) acc -= li[c2] * Lj[c2];
                Si[j] = acc;
            }
        }
        __syncthreads();
    }
    return s.ok != 0;
}

// Solve L L^T x = b in place in FP32 by warp 0 alone (no block barriers): lane l holds rows
// l + 32 q, q < kSolveRows (m <= 32 kSolveRows); the owner of row j finalizes x_j and broadcasts it.
constexpr int kSolveRows = 5;
static_assert(6 * kWinMaxFreeCams <= 32 * kSolveRows, "reduced system larger than the warp solve");
__device__ void warp_chol_solve32(const float* L, const float* rinv, int m, float* x) {
    if (threadIdx.x >= 32) return;
    const int lane = threadIdx.x;
    float xr[kSolveRows], rr[kSolveRows];  // the lane's rows of x and their 1/L_jj (off the serial chain)
#pragma unroll
    for (int q = 0; q < kSolveRows; ++q) {
        xr[q] = lane + 32 * q < m ? x[lane + 32 * q] : 0.f;
        rr[q] = lane + 32 * q < m ? rinv[lane + 32 * q] : 1.f;
    }
#pragma unroll
    for (int q = 0; q < kSolveRows; ++q) {
        for (int jj = 0; jj < 32; ++jj) {
            const int j = 32 * q + jj;
            if (j >= m) break;
            if (lane == jj) xr[q] *= rr[q];
            const float xj = __shfl_sync(kFull, xr[q], jj);
#pragma unroll
            for (int qq = q; qq < kSolveRows; ++qq) {
                const int i = lane + 32 * qq;
                if (i > j && i < m) xr[qq] -= L[tri(i, j)] * xj;
            }
        }
    }
#pragma unroll
    for (int q = kSolveRows - 1; q >= 0; --q) {
        for (int jj = 31; jj >= 0; --jj) {
            const int j = 32 * q + jj;
            if (j >= m) continue;
            if (lane == jj) xr[q] *= rr[q];
            const float xj = __shfl_sync(kFull, xr[q], jj);
            const float* Lj = L + tri(j, 0);
#pragma unroll
            for (int qq = 0; qq <= q; ++qq) {
                const int i = lane + 32 * qq;
                if (i < j) xr[qq] -= Lj[i] * xj;
            }
        }
    }
#pragma unroll
    for (int q = 0; q < kSolveRows; ++q)
        if (lane + 32 * q < m) x[lane + 32 * q] = xr[q];
}

// Mixed form: solve S x = b (x into b) with the Cholesky factor of S rounded to FP32 and one
// refinement step against the FP64 S: x0 from the FP32 factor, r = b - S x0 in FP64, x = x0 +
// (the FP32 factor's solution of r).  S's entries are FP32 sums already, so the FP32 factor adds
// an error of the same order, which the refinement step removes.  When the FP32 factorization
// meets a pivot that is not positive, S is factored in FP64 (S is kept intact for this).
// Returns false if S is not positive definite in FP64 either.  mark(k): phase-timer marks.
template <class Mark>
__device__ bool solve_s_mixed(double* S, double* rinv, float* S32, float* v32, int m, SmemHead& s, double* b,
                              Mark&& mark) {
    float* r32 = v32;           // 1/L_jj
    float* x32 = v32 + m;       // x0
    float* y32 = v32 + 2 * m;   // correction
    // S32 holds S rounded to FP32 already (written beside S by the block write-back)
    for (int k = threadIdx.x; k < m; k += blockDim.x) x32[k] = (float)b[k];
    __syncthreads();
    const bool ok32 = smem_cholesky_blocked(S32, r32, m, s);
    __syncthreads();  // every thread has read the outcome before s.ok is used again
    mark(10);
    if (!ok32) {
        if (!smem_cholesky<double>(S, rinv, m, s)) return false;
        smem_chol_solve(S, rinv, m, b);
        return true;
    }
    warp_chol_solve32(S32, r32, m, x32);
    __syncthreads();
    mark(11);
    // r = b - S x0, thread per row (row i of the packed lower S, then column i below it); x0 is
    // widened to FP64 once, into rinv (unused on this path)
    double* x0 = rinv;
    for (int k = threadIdx.x; k < m; k += blockDim.x) x0[k] = (double)x32[k];
    __syncthreads();
    for (int i = threadIdx.x; i < m; i += blockDim.x) {
        double acc = b[i];
        const double* Si = S + tri(i, 0);
        for (int k = 0; k <= i; ++k) acc -= Si[k] * x0[k];
        for (int k = i + 1; k < m; ++k) acc -= S[tri(k, i)] * x0[k];
        y32[i] = (float)acc;
    }
    __syncthreads();
    mark(12);
    warp_chol_solve32(S32, r32, m, y32);
    __syncthreads();
    mark(11);
    for (int k = threadIdx.x; k < m; k += blockDim.x) b[k] = x0[k] + (double)y32[k];
    __syncthreads();
    return true;
}

// Phase timer: thread 0 of rank 0 adds the SM cycles since the previous mark to phase `ph`.
struct PhaseClock {
    unsigned long long* acc;
    long long last;
    __device__ PhaseClock(unsigned long long* a, const CC& c) : acc(c.rank == 0 && threadIdx.x == 0 ? a : nullptr) {
        last = clock64();
    }
    __device__ __forceinline__ void mark(int ph) {
        if (!acc) return;
        const long long now = clock64();
        atomicAdd(acc + ph, (unsigned long long)(now - last));
        last = now;
    }
};

template <class Real>
__device__ void solve_window(const WinArgs<Real>& A, CC& c, int w, unsigned char* smem) {
    SmemHead& s = *c.s;
    PhaseClock pc(A.phase, c);
    const WinDesc D = A.win[w];
    const int m = 6 * D.nfc;
    const Dyn dl = dyn_layout(A.max_m, A.max_ncam, (int)sizeof(Real));
    CamState* cams0 = reinterpret_cast<CamState*>(smem + dl.cams);
    CamState* cams1 = cams0 + A.max_ncam;
    Real* camr = reinterpret_cast<Real*>(smem + dl.camr);
    Real* camr_tr = camr + 12 * A.max_ncam;
    double* camd = reinterpret_cast<double*>(smem + dl.camd);  // FP64 copies for the cost (mixed form)
    double* camd_tr = camd + 12 * A.max_ncam;
    Real* camdel = reinterpret_cast<Real*>(smem + dl.camdel);  // trial step per camera: E - I, E_t
    double* dcl = reinterpret_cast<double*>(smem + dl.dcl);
    Real* dclr = reinterpret_cast<Real*>(smem + dl.dclr);  // dcl rounded to Real
    double* S_smem = reinterpret_cast<double*>(smem + dl.S);
    // the reduced system: rank 0's shared memory (FP64 form) or the window's global scratch (mixed
    // form: it is read only by the refinement residual and the FP64 fallback; the FP32 factor is
    // in shared memory), written by every rank of the cluster
    double* S = sizeof(Real) == 4 ? A.s_glob + D.s0 : S_smem;
    if (sizeof(Real) == 4) c.S0 = S;
    double* bs = reinterpret_cast<double*>(smem + dl.bs);
    double* rinv = reinterpret_cast<double*>(smem + dl.rinv);
    float* S32 = reinterpret_cast<float*>(smem + dl.s32);
    float* v32 = reinterpret_cast<float*>(smem + dl.v32);
    WinStats* st = A.stats + w;
    double* trace = A.trace + (long long)w * A.trace_stride;
    const bool mixed = sizeof(Real) == 4;
    // mixed form, pinhole model: trial costs as the FP64 current cost plus FP32 residual changes
    // (update_points_dcost); otherwise every trial cost is evaluated in FP64
    const bool dcost = mixed && A.edge_e[0] != nullptr && A.intr.model == 0;

    for (int k = threadIdx.x; k < D.ncam; k += blockDim.x) {
        cams0[k] = A.cam_init[D.cam0 + k];
        cams1[k] = A.cam_init[D.cam0 + k];
        cam_real<Real>(cams0[k], camr + 12 * k);
        cam_real<Real>(cams0[k], camr_tr + 12 * k);
        cam_real<double>(cams0[k], camd + 12 * k);
        cam_real<double>(cams0[k], camd_tr + 12 * k);
    }
    for (int p = c.gt; p < D.npt; p += c.CT) {
        const long long gp = D.pt0 + p;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            A.x[0][4 * gp + k] = A.pt_init[4 * gp + k];
            A.x[1][4 * gp + k] = A.pt_init[4 * gp + k];
            if (A.xr[0]) {
                A.xr[0][4 * gp + k] = (Real)A.pt_init[4 * gp + k];
                A.xr[1][4 * gp + k] = (Real)A.pt_init[4 * gp + k];
            }
        }
    }
    if (A.edge_uvr)
        for (int e = c.gt; e < 2 * D.ne; e += c.CT) A.edge_uvr[2LL * D.e0 + e] = (Real)A.edge_uv[2LL * D.e0 + e];
    if (threadIdx.x == 0) s.cur = 0;
    if (c.rank == 0 && threadIdx.x == 0) st->depth_nonpos = 0;  // summed by every warp at the end
    __syncthreads();
    pc.mark(13);
    // the camera-list counting sort's per-warp table borrows the S region (unused until the first
    // trial; dyn_layout sizes it for the table)
    build_lists(A, c, D, reinterpret_cast<int32_t(*)[kWinMaxCams]>(S_smem), [&](int k) { pc.mark(k); });  // ends with a cluster barrier: points are initialized everywhere
    pc.mark(0);

    // the initial cost is FP64 in both forms; the FP64 form evaluates every trial cost in FP64, the
    // mixed form tracks FP32 residuals from these FP64 ones and sums the residual changes
    double chi = cluster_reduce3<false>(
        c, cost_partial<double, Real>(A, c, D, camd, A.x[0], dcost ? A.edge_e[0] : nullptr), 0.0, 0.0).x;
    const double chi0_fp64 = chi;
    int iters_done = 0, acc = 0, rej = 0, term = NAV_BA_TERM_ITERATIONS;
    double lambda = 0.0, nu = 2.0;
    pc.mark(1);
    if (c.rank == 0 && threadIdx.x == 0) trace[0] = chi;
    const bool bad = !isfinite(chi);
    if (!bad && D.nfc + D.nfp == 0) term = NAV_BA_TERM_NOTHING_TO_DO;
    if (!bad && term == NAV_BA_TERM_ITERATIONS) {
        for (int it = 0; it < A.lm.iterations; ++it) {
            const int cur = s.cur;
            Real* cr_cur = cur == 0 ? camr : camr_tr;
            const double mxp = linearize_points<Real>(A, c, D, cr_cur, A.x[cur], A.xr[cur]);
            pc.mark(2);
            const double mxc = linearize_cameras<Real>(A, c, D, cr_cur, A.x[cur], A.xr[cur]);
            const double maxdiag = cluster_reduce3<true>(c, fmax(mxp, mxc), 0.0, 0.0).x;
            pc.mark(3);
            if (it == 0) {
                lambda = A.lm.initial_lambda > 0 ? A.lm.initial_lambda : A.lm.tau * maxdiag;
                nu = 2.0;
            }
            double rho = 0.0;
            int q = 0;
            do {
                const double lam_use = (A.debug && it == 0 && q == 0) ? A.debug_lambda : lambda;
                if (c.rank == 0)
                    for (int k = threadIdx.x; k < m * (m + 1) / 2; k += blockDim.x) {
                        S[k] = 0.0;
                        if (mixed) S32[k] = 0.f;
                    }
                if (threadIdx.x == 0) s.next_blk = 0;  // ordered before the blocks by the reduction's barriers
                const int npd = schur_points<Real>(A, c, D, lam_use, cr_cur, A.x[cur], A.xr[cur]);
                const double3 r0 = cluster_reduce3<false>(c, (double)npd, 0.0, 0.0);  // also orders S zeroing
                pc.mark(4);
                schur_blocks<Real>(A, c, D, lam_use);
                csync(c);
                pc.mark(5);
                if (A.debug) {
                    if (c.rank == 0) {
                        for (int k = threadIdx.x; k < m * m; k += blockDim.x) {
                            const int r = k / m, cc = k % m;
                            A.debug[k] = r >= cc ? S[tri(r, cc)] : S[tri(cc, r)];
                        }
                        for (int k = threadIdx.x; k < m; k += blockDim.x) A.debug[m * m + k] = bs[k];
                    }
                    csync(c);
                    return;
                }
                if (c.rank == 0) {
                    bool okc;
                    if (mixed) {
                        okc = solve_s_mixed(S, rinv, S32, v32, m, s, bs, [&](int k) { pc.mark(k); }) && r0.x == 0.0;
                    } else {
                        okc = smem_cholesky<double>(S, rinv, m, s) && r0.x == 0.0;
                        if (okc) smem_chol_solve(S, rinv, m, bs);
                    }
                    if (!okc) {
                        for (int k = threadIdx.x; k < m; k += blockDim.x) bs[k] = 0.0;
                    }
                    __syncthreads();
                    if (threadIdx.x == 0) s.ok = okc ? 1 : 0;
                }
                csync(c);
                pc.mark(6);
                // every CTA takes the camera step from rank 0 and updates all cameras itself
                for (int k = threadIdx.x; k < m; k += blockDim.x) {
                    dcl[k] = c.bs0[k];
                    dclr[k] = (Real)dcl[k];
                }
                __syncthreads();
                const bool ok = c.s0->ok != 0;
                CamState* ccur = cur == 0 ? cams0 : cams1;
                CamState* ctr = cur == 0 ? cams1 : cams0;
                Real* crt = cur == 0 ? camr_tr : camr;
                double* cdt = cur == 0 ? camd_tr : camd;
                double sc = 0.0;
                for (int k = threadIdx.x; k < D.ncam; k += blockDim.x) {
                    const int a = A.cam_free[D.cam0 + k];
                    if (a >= 0) {
                        se3_left_update(dcl + 6 * a, ccur[k], ctr[k]);
                        if (c.rank == 0)
#pragma unroll
                            for (int r = 0; r < 6; ++r) sc += dcl[6 * a + r] * (lambda * dcl[6 * a + r] + s.U[a][21 + r]);
                    }
                    if (dcost) {
                        double emi[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0}, et[3] = {0, 0, 0};
                        if (a >= 0) se3_exp_delta(dcl + 6 * a, emi, et);
#pragma unroll
                        for (int r = 0; r < 9; ++r) camdel[12 * k + r] = (Real)emi[r];
#pragma unroll
                        for (int r = 0; r < 3; ++r) camdel[12 * k + 9 + r] = (Real)et[r];
                    }
                    cam_real<Real>(ctr[k], crt + 12 * k);
                    cam_real<double>(ctr[k], cdt + 12 * k);
                }
                __syncthreads();
                double chi_new, scale;
                if (dcost) {
                    const double2 ud = update_points_dcost<Real>(A, c, D, lambda, dclr, cur, cr_cur, camdel);
                    pc.mark(7);
                    const double3 red = cluster_reduce3<false>(c, ud.y, sc + ud.x, 0.0);
                    chi_new = chi + red.x;
                    scale = red.y;
                } else {
                    sc += update_points<Real>(A, c, D, lambda, dclr, cur);
                    pc.mark(7);
                    const double3 red = cluster_reduce3<false>(
                        c, cost_partial<double, Real>(A, c, D, cdt, A.x[cur ^ 1]), sc, 0.0);
                    chi_new = red.x;
                    scale = red.y;
                }
                // the decision is scalar FP64 work (a pow among it): one thread makes it, the others
                // read it, so the FP64 pipe is not charged once per thread
                if (threadIdx.x == 0) {
                    if (!ok) chi_new = DBL_MAX;
                    double r = chi - chi_new;
                    scale += 1e-3;
                    r /= scale;
                    // a failed damped system is a rejected trial (as g2o's DBL_MAX trial cost makes
                    // it), also when failed point blocks left the step scale non-finite
                    if (!ok) r = -DBL_MAX;
                    const bool accept = r > 0 && isfinite(chi_new);
                    double lam = lambda, n2 = nu, ch = chi;
                    if (accept) {
                        double alpha = 1.0 - pow(2 * r - 1, 3.0);
                        alpha = fmin(alpha, 2.0 / 3.0);
                        lam *= fmax(1.0 / 3.0, alpha);
                        n2 = 2.0;
                        ch = chi_new;
                        s.cur = cur ^ 1;
                    } else {
                        lam *= n2;
                        n2 *= 2;
                    }
                    s.lm[0] = r;
                    s.lm[1] = lam;
                    s.lm[2] = n2;
                    s.lm[3] = ch;
                    s.lm_acc = accept;
                }
                __syncthreads();
                rho = s.lm[0];
                lambda = s.lm[1];
                nu = s.lm[2];
                chi = s.lm[3];
                if (s.lm_acc) ++acc; else ++rej;
                __syncthreads();  // the decision is read before the next trial overwrites it
                pc.mark(8);
                ++q;
            } while (rho < 0 && q < A.lm.max_trials);
            iters_done = it + 1;
            if (c.rank == 0 && threadIdx.x == 0) trace[it + 1] = chi;
            if (q == A.lm.max_trials) { term = NAV_BA_TERM_TRIALS_EXHAUSTED; break; }
            if (rho == 0) { term = NAV_BA_TERM_ZERO_GAIN; break; }
            if (!isfinite(lambda)) { term = NAV_BA_TERM_LAMBDA_NONFINITE; break; }
        }
    }
    const int cur = s.cur;
    CamState* cfin = cur == 0 ? cams0 : cams1;
    double chi_final = chi;
    if (dcost && !bad) {
        // the final cost reported is the FP64 cost of the final state
        chi_final = cluster_reduce3<false>(c, cost_partial<double, Real>(A, c, D, cur == 0 ? camd : camd_tr, A.x[cur]),
                                           0.0, 0.0).x;
        if (c.rank == 0 && threadIdx.x == 0) trace[iters_done] = chi_final;
    }
    if (c.rank == 0)
        for (int k = threadIdx.x; k < D.ncam; k += blockDim.x) A.cam_out[D.cam0 + k] = cfin[k];
    // the final points out, and the active edges whose point is at or behind its camera
    int nneg = 0;
    for (int p = c.gt; p < D.npt; p += c.CT) {
        const long long gp = D.pt0 + p;
        double X[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            X[k] = A.x[cur][4 * gp + k];
            A.pt_out[4 * gp + k] = X[k];
        }
        const int e1 = A.pt_eoff[gp + 1];
        for (int e = A.pt_eoff[gp]; e < e1; ++e) nneg += depth_nonpositive(cfin[A.edge_cam[e]], X) ? 1 : 0;
    }
    nneg = __reduce_add_sync(kFull, nneg);
    if (c.lane == 0 && nneg) atomicAdd(&st->depth_nonpos, nneg);
    if (c.rank == 0 && threadIdx.x == 0) {
        st->initial_cost = chi0_fp64;
        st->final_cost = chi_final;
        st->final_lambda = lambda;
        st->iterations_done = iters_done;
        st->accepted = acc;
        st->rejected = rej;
        st->termination = term;
        st->status = bad ? NAV_BA_ERR_NONFINITE_COST : NAV_BA_OK;
    }
    csync(c);
    pc.mark(9);
}

// The view of CTA `rank` of `csize` CTAs sharing one window (rank 0's shared memory holds the
// window's reduced system and head; csize 1: the CTA alone).  f32: the mixed form, whose rank 0
// also keeps the FP32 copy of the reduced system.
__device__ CC make_view(unsigned char* smem_raw, int rank, int csize, const Dyn& dl, bool f32) {
    CC c;
    c.rank = rank;
    c.csize = csize;
    c.lane = threadIdx.x & 31;
    c.wid = threadIdx.x >> 5;
    c.nw = blockDim.x >> 5;
    c.gt = c.rank * blockDim.x + threadIdx.x;
    c.CT = c.csize * blockDim.x;
    c.gw = c.rank * c.nw + c.wid;
    c.CW = c.csize * c.nw;
    c.s = reinterpret_cast<SmemHead*>(smem_raw);
    c.s0 = c.s;
    c.S0 = reinterpret_cast<double*>(smem_raw + dl.S);
    c.bs0 = reinterpret_cast<double*>(smem_raw + dl.bs);
    c.S0f = f32 ? reinterpret_cast<float*>(smem_raw + dl.s32) : nullptr;
    if (csize > 1) {
        cg::cluster_group cl = cg::this_cluster();
        c.s0 = cl.map_shared_rank(c.s, 0);
        c.S0 = cl.map_shared_rank(c.S0, 0);
        c.bs0 = cl.map_shared_rank(c.bs0, 0);
        if (f32) c.S0f = cl.map_shared_rank(c.S0f, 0);
    }
    return c;
}

// Per-window schedule: the first A.n_big windows of the queue (the largest, host-ordered) are each
// solved by a whole cluster, which cuts their latency (they set the launch's critical path); once
// that part of the queue is taken, every CTA of the cluster takes the remaining windows one at a
// time from a second queue and solves each alone (no cluster barriers, no distributed shared
// memory).  A launch with clusters of one CTA solves every window alone.
template <class Real>
__global__ void __launch_bounds__(sizeof(Real) == 8 ? 256 : 512) window_lm_kernel(WinArgs<Real> A) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cg::cluster_group cl = cg::this_cluster();
    const Dyn dl = dyn_layout(A.max_m, A.max_ncam, (int)sizeof(Real));
    const int csize = (int)cl.num_blocks();
    SmemHead* head = reinterpret_cast<SmemHead*>(smem_raw);
    if (threadIdx.x == 0) head->slot = 0;
    __syncthreads();
    // one call site of solve_window (a second inlined copy costs registers)
    bool clustered = csize > 1;
    CC c = make_view(smem_raw, clustered ? (int)cl.block_rank() : 0, csize, dl, sizeof(Real) == 4);
    for (;;) {
        int w;
        if (clustered) {
            if (c.rank == 0 && threadIdx.x == 0) {
                const int k = atomicAdd(A.queue, 1);
                c.s->win = k < A.n_big ? A.order[k] : -1;
            }
            csync(c);
            w = c.s0->win;
            csync(c);  // every rank has read rank 0's window index
            if (w < 0) {
                if (A.debug) return;
                // the clusters' part of the queue is done: from here on every CTA works alone, and
                // nothing reads another CTA's shared memory any more
                clustered = false;
                c = make_view(smem_raw, 0, 1, dl, sizeof(Real) == 4);
                continue;
            }
        } else {
            if (threadIdx.x == 0) {
                const int k = (csize > 1 ? A.n_big : 0) + atomicAdd(A.queue + 1, 1);
                c.s->win = k < A.n_win ? A.order[k] : -1;
            }
            __syncthreads();
            w = c.s->win;
            __syncthreads();
            if (w < 0) break;
        }
        solve_window<Real>(A, c, w, smem_raw);
        if (A.debug) break;
    }
    if (clustered) csync(c);  // a cluster that stopped early (debug) leaves together
}

template <class Real>
cudaError_t launch_typed(PreparedBatch& pb, cudaStream_t stream, WindowLaunch shape, double debug_lambda) {
    WindowBatch& b = pb.dev;
    WinArgs<Real> A{};  // every field not set below stays null or zero
    A.win = b.d_win;
    A.n_win = b.n_queue;
    // the windows solved by whole clusters: the leading ones of weight >= big_weight
    A.n_big = 0;
    if (shape.cluster > 1) {
        const auto& ow = b.order_weight;
        const int n_w = std::min<int>((int)ow.size(), b.n_queue);
        while (A.n_big < n_w && ow[A.n_big] >= shape.big_weight) ++A.n_big;
        if (ow.empty()) A.n_big = b.n_queue;
    }
    if (debug_lambda >= 0) A.n_big = b.n_queue;  // the reduced system of window 0, by one cluster
    A.order = b.d_order;
    A.queue = b.d_queue;
    A.cam_init = b.d_cam_init;
    A.cam_free = b.d_cam_free;
    A.pt_init = b.d_pt_init;
    A.pt_free = b.d_pt_free;
    A.pt_eoff = b.d_pt_eoff;
    A.edge_cam = b.d_edge_cam;
    A.edge_fc = b.d_edge_fc;
    A.edge_pt = b.d_edge_pt;
    A.edge_uv = b.d_edge_uv;
    A.edge_uvr = sizeof(Real) == 4 ? (Real*)b.d_edge_uvr : nullptr;
    A.x[0] = b.d_x[0];
    A.x[1] = b.d_x[1];
    A.xr[0] = sizeof(Real) == 4 ? (Real*)b.d_xr[0] : nullptr;
    A.xr[1] = sizeof(Real) == 4 ? (Real*)b.d_xr[1] : nullptr;
    A.pt_vg = (Real*)b.d_pt_vg;
    A.pt_lt = (Real*)b.d_pt_lt;
    A.edge_w = sizeof(Real) == 8 ? (Real*)b.d_edge_w : nullptr;
    A.edge_a = (Real*)b.d_edge_a;
    A.jfact = sizeof(Real) == 4 && pb.intr.model == 0;
    A.edge_e[0] = sizeof(Real) == 4 ? (Real*)b.d_edge_e[0] : nullptr;
    A.edge_e[1] = sizeof(Real) == 4 ? (Real*)b.d_edge_e[1] : nullptr;
    A.cam_list = b.d_cam_list;
    A.s_glob = sizeof(Real) == 4 ? b.d_s : nullptr;
    A.pairs = b.d_pairs;
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
    A.max_ncam = std::max(1, b.max_ncam);
    A.phase = b.d_phase;
    if (b.d_phase) cudaMemsetAsync(b.d_phase, 0, sizeof(unsigned long long) * kWinPhases, stream);
    const int C = std::max(1, std::min(kMaxCluster, shape.cluster));
    const int T = shape.threads;
    if (T % 32 != 0 || T < 64 || T > (sizeof(Real) == 8 ? 256 : 512)) return cudaErrorInvalidConfiguration;
    const size_t smem = dyn_layout(A.max_m, A.max_ncam, (int)sizeof(Real)).total;
    const void* kern = (const void*)window_lm_kernel<Real>;
    cudaError_t err = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (err != cudaSuccess) return err;
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = C;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cfg.blockDim = dim3(T);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = stream;
    int max_clusters = 0;
    cfg.gridDim = dim3(C);
    err = cudaOccupancyMaxActiveClusters(&max_clusters, kern, &cfg);
    if (err != cudaSuccess) return err;
    if (max_clusters < 1) return cudaErrorInvalidConfiguration;
    int clusters = std::min(max_clusters, b.n_queue);
    if (debug_lambda >= 0) clusters = 1;
    cfg.gridDim = dim3(clusters * C);
    err = cudaMemsetAsync(b.d_queue, 0, 2 * sizeof(int32_t), stream);
    if (err != cudaSuccess) return err;
    void* args[] = {&A};
    return cudaLaunchKernelExC(&cfg, kern, args);
}

}  // namespace

size_t window_smem_bytes(int max_m, int max_ncam, int precision) {
    return dyn_layout(max_m, std::max(1, max_ncam), precision == NAV_BA_MIXED ? 4 : 8).total;
}

cudaError_t window_batch_launch(PreparedBatch& pb, cudaStream_t stream, int precision, WindowLaunch shape,
                                double debug_lambda) {
    if (pb.dev.n_queue == 0) return cudaSuccess;
    if (precision == NAV_BA_MIXED) return launch_typed<float>(pb, stream, shape, debug_lambda);
    return launch_typed<double>(pb, stream, shape, debug_lambda);
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
        const Intr in = make_intr(p.intrinsics, p.camera_model);
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

// Work weight of a window for the schedule: edges, Schur pairs and a Cholesky-size term.
static double window_weight(const HostWindow& h) {
    return (double)h.ne + (double)h.n_pairs + 2.0 * h.nfc * h.nfc * h.nfc;
}

void* HostStaging::get(int id, size_t bytes) {
    bytes = std::max<size_t>(bytes, 64);
    if (cap[id] >= bytes) return buf[id];
    if (buf[id]) cudaFreeHost(buf[id]);
    buf[id] = nullptr;
    cap[id] = 0;
    const size_t want = bytes + bytes / 4;
    if (cudaHostAlloc(&buf[id], want, cudaHostAllocDefault) != cudaSuccess) {
        buf[id] = nullptr;
        return nullptr;
    }
    cap[id] = want;
    return buf[id];
}

void HostStaging::release() {
    for (int i = 0; i < 16; ++i) {
        if (buf[i]) cudaFreeHost(buf[i]);
        buf[i] = nullptr;
        cap[i] = 0;
    }
}

void window_batch_free(WindowBatch& b) {
    void* ptrs[] = {b.d_win, b.d_order, b.d_queue, b.d_cam_init, b.d_cam_free, b.d_pt_init, b.d_pt_free,
                    b.d_pt_eoff, b.d_edge_cam, b.d_edge_fc, b.d_edge_pt, b.d_edge_uv, b.d_x[0], b.d_x[1], b.d_pt_vg,
                    b.d_pt_lt, b.d_edge_w, b.d_edge_a, b.d_edge_e[0], b.d_edge_e[1], b.d_cam_list, b.d_pairs, b.d_edge_uvr, b.d_s, b.d_xr[0], b.d_xr[1], b.d_cam_out, b.d_pt_out,
                    b.d_trace, b.d_stats, b.d_debug, b.d_phase};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    b = WindowBatch();
}

namespace {

// Run fn(i) for i in [0, n) on the context's host workers (contiguous chunks).
template <class Fn>
void parallel_for(HostPool& pool, int n, Fn fn) {
    const int nt = HostPool::tasks_for(n, 4);
    pool.run(nt, [&](int t) {
        const int lo = (int)((long long)n * t / nt), hi = (int)((long long)n * (t + 1) / nt);
        for (int i = lo; i < hi; ++i) fn(i);
    });
}

// Per-edge arrays derived on the device from what is uploaded (8 of the 36 bytes an observation
// would otherwise take on the bus): the window-local point of each edge (edges are point-major,
// pt_eoff holds the global offsets) and its free-camera index.  Block per chunk of a window's
// points, thread per point.
constexpr int kEdgeDeriveChunk = 1024;
__global__ void k_edge_derive(const WinDesc* win, int nw, int nchunk, const int32_t* pt_eoff, const int32_t* edge_cam,
                              const int32_t* cam_free, int32_t* edge_pt, int32_t* edge_fc) {
    // block b: chunk b % nchunk of window b / nchunk (kEdgeDeriveChunk points per chunk)
    for (int b = blockIdx.x; b < nw * nchunk; b += gridDim.x) {
        const WinDesc d = win[b / nchunk];
        const int k1 = min(d.npt, (b % nchunk + 1) * kEdgeDeriveChunk);
        for (int k = (b % nchunk) * kEdgeDeriveChunk + threadIdx.x; k < k1; k += blockDim.x) {
            const int e0 = pt_eoff[d.pt0 + k];
            const int e1 = k + 1 < d.npt ? pt_eoff[d.pt0 + k + 1] : d.e0 + d.ne;
            for (int e = e0; e < e1; ++e) {
                edge_pt[e] = k;
                edge_fc[e] = cam_free[d.cam0 + edge_cam[e]];
            }
        }
    }
}

}  // namespace

cudaError_t window_batch_upload(PreparedBatch& pb, cudaStream_t stream, int precision, int trace_stride,
                                HostStaging& stg, HostPool& pool, std::string* why, bool sync) {
    WindowBatch& b = pb.dev;
    std::vector<int32_t> idx;
    for (size_t i = 0; i < pb.host.size(); ++i)
        if (pb.host_status[i] == NAV_BA_OK) idx.push_back((int32_t)i);
    pb.desc.assign(pb.host.size(), WinDesc{});
    int64_t nc = 0, np = 0, ne = 0, npair = 0, ns = 0;
    int max_m = 0, max_nc = 0, max_npt = 0;
    for (size_t i = 0; i < pb.host.size(); ++i) {
        const HostWindow& h = pb.host[i];
        WinDesc& d = pb.desc[i];
        d.cam0 = (int32_t)nc; d.ncam = h.ncam;
        d.pt0 = (int32_t)np; d.npt = h.npt;
        d.e0 = (int32_t)ne; d.ne = h.ne;
        d.nfc = h.nfc; d.nfp = h.nfp;
        d.pair0 = npair; d.npair = h.n_pairs;
        d.s0 = ns;
        nc += h.ncam; np += h.npt; ne += h.ne; npair += h.n_pairs;
        max_npt = std::max(max_npt, h.npt);
        ns += (int64_t)(6 * h.nfc) * (6 * h.nfc + 1) / 2;
        if (pb.host_status[i] == NAV_BA_OK) {
            max_m = std::max(max_m, 6 * h.nfc);
            max_nc = std::max(max_nc, h.ncam);
        }
    }
    if (nc > INT32_MAX || np > INT32_MAX || ne > INT32_MAX - 1) {
        if (why) *why = "batch too large for 32-bit indices";
        return cudaErrorInvalidValue;
    }
    // schedule: largest windows first (edges, pairs and a Cholesky-size term)
    std::vector<int32_t> order = idx;
    std::stable_sort(order.begin(), order.end(), [&](int32_t x, int32_t y) {
        return window_weight(pb.host[x]) > window_weight(pb.host[y]);
    });
    b.order_weight.resize(order.size());
    for (size_t k = 0; k < order.size(); ++k) b.order_weight[k] = window_weight(pb.host[order[k]]);
    const size_t rs = real_size(precision);
    const size_t nw = pb.desc.size();
    cudaError_t err = cudaSuccess;
    int slot = 0;
    b.bytes = 0;
    auto ensure = [&](auto** p, size_t bytes) {
        const int id = slot++;
        if (err != cudaSuccess) return;
        bytes = std::max<size_t>(bytes, 16);
        b.bytes += bytes;
        if (*p && b.cap[id] >= bytes) return;
        if (*p) cudaFree(*p);
        *p = nullptr;
        b.cap[id] = 0;
        err = cudaMalloc((void**)p, bytes);
        if (err == cudaSuccess) b.cap[id] = bytes;
    };
    ensure(&b.d_win, sizeof(WinDesc) * nw);
    ensure(&b.d_order, sizeof(int32_t) * order.size());
    ensure(&b.d_queue, 2 * sizeof(int32_t));
    ensure(&b.d_cam_init, sizeof(CamState) * nc);
    ensure(&b.d_cam_free, sizeof(int32_t) * nc);
    ensure(&b.d_pt_init, sizeof(double) * 4 * np);
    ensure(&b.d_pt_free, sizeof(int32_t) * np);
    ensure(&b.d_pt_eoff, sizeof(int32_t) * (np + 1));
    ensure(&b.d_edge_cam, sizeof(int32_t) * ne);
    ensure(&b.d_edge_fc, sizeof(int32_t) * ne);
    ensure(&b.d_edge_pt, sizeof(int32_t) * ne);
    ensure(&b.d_edge_uv, sizeof(double) * 2 * ne);
    ensure(&b.d_x[0], sizeof(double) * 4 * np);
    ensure(&b.d_x[1], sizeof(double) * 4 * np);
    ensure(&b.d_pt_vg, rs * 12 * np);
    ensure(&b.d_pt_lt, rs * 12 * np);
    const size_t rec = precision == NAV_BA_MIXED ? 20 : 18;  // per-edge record stride (Reals)
    ensure(&b.d_edge_w, precision == NAV_BA_MIXED ? 16 : rs * rec * ne);  // FP64 form only
    ensure(&b.d_edge_a, rs * rec * ne);
    ensure(&b.d_edge_e[0], precision == NAV_BA_MIXED ? rs * 2 * ne : 16);
    ensure(&b.d_edge_e[1], precision == NAV_BA_MIXED ? rs * 2 * ne : 16);
    ensure(&b.d_cam_list, sizeof(int32_t) * ne);
    ensure(&b.d_pairs, sizeof(uint32_t) * npair);
    ensure(&b.d_edge_uvr, precision == NAV_BA_MIXED ? rs * 2 * ne : 16);  // mixed form only
    ensure(&b.d_s, precision == NAV_BA_MIXED ? sizeof(double) * ns : 16);
    ensure(&b.d_xr[0], precision == NAV_BA_MIXED ? rs * 4 * np : 16);
    ensure(&b.d_xr[1], precision == NAV_BA_MIXED ? rs * 4 * np : 16);
    ensure(&b.d_cam_out, sizeof(CamState) * nc);
    ensure(&b.d_pt_out, sizeof(double) * 4 * np);
    ensure(&b.d_trace, sizeof(double) * trace_stride * nw);
    ensure(&b.d_stats, sizeof(WinStats) * nw);
    ensure(&b.d_debug, sizeof(double) * ((size_t)max_m * max_m + max_m));
    const char* pt_env = getenv("NAVBA_PHASE_TIMING");
    if (pt_env && pt_env[0] == '1') {
        ensure(&b.d_phase, sizeof(unsigned long long) * kWinPhases);
    } else {
        if (b.d_phase) cudaFree(b.d_phase);
        b.d_phase = nullptr;
        b.cap[slot++] = 0;
    }
    if (err != cudaSuccess) {
        if (why) *why = cudaGetErrorString(err);
        return err;
    }
    b.n_win = (int32_t)nw;
    b.ncam = nc; b.npt = np; b.ne = ne; b.npair = npair;
    b.max_m = max_m;
    b.max_ncam = max_nc;
    b.precision = precision;
    b.trace_stride = trace_stride;
    // stage the concatenated inputs in pinned memory (parallel over windows), then copy
    CamState* cam = (CamState*)stg.get(0, sizeof(CamState) * nc);
    int32_t* cam_free = (int32_t*)stg.get(1, sizeof(int32_t) * nc);
    double* pt = (double*)stg.get(2, sizeof(double) * 4 * np);
    int32_t* pt_free = (int32_t*)stg.get(3, sizeof(int32_t) * np);
    int32_t* pt_eoff = (int32_t*)stg.get(4, sizeof(int32_t) * (np + 1));
    int32_t* edge_cam = (int32_t*)stg.get(5, sizeof(int32_t) * ne);
    double* uv = (double*)stg.get(7, sizeof(double) * 2 * ne);
    WinDesc* desc = (WinDesc*)stg.get(8, sizeof(WinDesc) * nw);
    int32_t* ord = (int32_t*)stg.get(9, sizeof(int32_t) * order.size());
    if (!cam || !cam_free || !pt || !pt_free || !pt_eoff || !edge_cam || !uv || !desc || !ord) {
        if (why) *why = "pinned host allocation failed";
        return cudaErrorMemoryAllocation;
    }
    std::copy(pb.desc.begin(), pb.desc.end(), desc);
    std::copy(order.begin(), order.end(), ord);
    parallel_for(pool, (int)nw, [&](int i) {
        const HostWindow& h = pb.host[i];
        const WinDesc& d = pb.desc[i];
        std::copy(h.cam.begin(), h.cam.end(), cam + d.cam0);
        std::copy(h.cam_free.begin(), h.cam_free.end(), cam_free + d.cam0);
        std::copy(h.pt_free.begin(), h.pt_free.end(), pt_free + d.pt0);
        std::copy(h.pt.begin(), h.pt.end(), pt + 4LL * d.pt0);
        for (int k = 0; k < h.npt; ++k) pt_eoff[d.pt0 + k] = d.e0 + h.pt_eoff[k];
        std::copy(h.edge_cam.begin(), h.edge_cam.end(), edge_cam + d.e0);
        std::copy(h.edge_uv.begin(), h.edge_uv.end(), uv + 2LL * d.e0);
    });
    pt_eoff[np] = (int32_t)ne;
    b.h2d_bytes = 0;
    auto up = [&](void* dst, const void* src, size_t bytes) {
        if (err != cudaSuccess || bytes == 0) return;
        err = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, stream);
        b.h2d_bytes += (int64_t)bytes;
    };
    up(b.d_win, desc, sizeof(WinDesc) * nw);
    up(b.d_order, ord, sizeof(int32_t) * order.size());
    up(b.d_cam_init, cam, sizeof(CamState) * nc);
    up(b.d_cam_free, cam_free, sizeof(int32_t) * nc);
    up(b.d_pt_init, pt, sizeof(double) * 4 * np);
    up(b.d_pt_free, pt_free, sizeof(int32_t) * np);
    up(b.d_pt_eoff, pt_eoff, sizeof(int32_t) * (np + 1));
    up(b.d_edge_cam, edge_cam, sizeof(int32_t) * ne);
    up(b.d_edge_uv, uv, sizeof(double) * 2 * ne);
    if (err == cudaSuccess && nw > 0) {
        // a block per chunk of a window's points: one large window (the grid engine's) spreads
        // over the GPU instead of running on one block (0.5 ms for 50k points)
        const int nchunk = std::max(1, (max_npt + kEdgeDeriveChunk - 1) / kEdgeDeriveChunk);
        k_edge_derive<<<(int)std::min<size_t>((size_t)nw * nchunk, 8192), 128, 0, stream>>>(
            b.d_win, (int)nw, nchunk, b.d_pt_eoff, b.d_edge_cam, b.d_cam_free, b.d_edge_pt, b.d_edge_fc);
        err = cudaGetLastError();
    }
    if (err == cudaSuccess && sync) err = cudaStreamSynchronize(stream);
    b.n_queue = (int32_t)order.size();
    if (err != cudaSuccess && why) *why = cudaGetErrorString(err);
    return err;
}

void window_phase_report(const PreparedBatch& pb, const WindowLaunch& shape, int precision) {
    if (!pb.dev.d_phase) return;
    unsigned long long h[kWinPhases] = {};
    if (cudaMemcpy(h, pb.dev.d_phase, sizeof(h), cudaMemcpyDeviceToHost) != cudaSuccess) return;
    static const char* names[kWinPhases] = {"lists: pair fill", "initial cost", "linearize points", "linearize cameras",
                                            "schur points", "schur blocks", "cholesky", "update", "trial cost",
                                            "outputs", "  chol: f32 factor", "  chol: f32 solves", "  chol: refine",
                                            "  init: states", "  lists: cameras", "  lists: pair counts"};
    unsigned long long tot = 0;
    for (int k = 0; k < kWinPhases; ++k) tot += h[k];
    fprintf(stderr, "[navba phases] precision=%d cluster=%d threads=%d total=%llu cycles (rank-0 CTAs, summed)\n",
            precision, shape.cluster, shape.threads, tot);
    for (int k = 0; k < kWinPhases; ++k)
        fprintf(stderr, "[navba phases] %-18s %14llu  %5.1f%%\n", names[k], h[k], tot ? 100.0 * h[k] / tot : 0.0);
}

}  // namespace navba
