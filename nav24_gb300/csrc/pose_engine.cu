// pose_engine.cu - motion-only BA (one free pose against fixed world points), many problems per
// launch, one block per problem.
//
// The edge is nav24's EdgeSE3ProjectXYZOnlyPose (core/dataTypes/optimization/OptimizableTypes.hpp:34-60,
// OptimizableTypes.cpp:50-64): e = z - pi(T Xw) with J = -Jpi [-[Xc]x | I], the same residual and pose
// Jacobian as the full edge with the point block dropped.  The LM control is the one of the other
// engines (g2o OptimizationAlgorithmLevenberg::solve semantics) on the 6x6 normal equations:
//   the block's threads stride over the problem's observations (structure of arrays: point [n][4],
//   uv [n][2]); H (21 packed) and b (6) accumulate per thread in Real and are summed in FP64 (a
//   warp reduce-scatter, then over the warps in order); thread 0 factors H + lambda I (FP64 Cholesky, in
//   registers), applies the SE(3) update and makes the LM decisions, which the block reads from
//   shared memory; costs are FP64 per-thread partial sums reduced the same way (fixed order:
//   bitwise repeatable).  A single frame is one block, not one warp: its dependent FP64 chains
//   (one warp: IPC 0.08, fixed-latency waits) overlap over eight warps.
#include <cfloat>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "engine.hpp"

namespace navba {
namespace {

constexpr unsigned kPoseFull = 0xffffffffu;

struct PoseArgs {
    const PoseDesc* desc;
    int n;
    const CamState* cam_in;
    CamState* cam_out;
    const double* pts;  // [no][4]
    const double* uv;   // [no][2]
    PoseStat* stats;
    LmOptions lm;
};

NAVBA_HD int ptri(int r, int c) { return r * (r + 1) / 2 + c; }

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kPoseFull, v, o);
    return v;
}

// Warp reduce-scatter of N <= 32 values per lane: lane k < N returns the warp's total of value k.
// Recursive halving over lane bits 4..0: at each level a lane keeps one half of its values (the
// upper when its lane bit is set) and adds its partner's copy of that half, so lane k ends with
// value k, summed over the same tree as warp_sum's butterfly (pairs across lane bit 4, then 3, ..
// 0) and equal to it bit for bit.  31 shuffles and FP64 adds per lane for all N values, against 5
// per value with a butterfly each: on GB300 an FP64 instruction occupies its SM partition 64
// cycles per warp, and the 27 butterflies of H and b were half of the mixed form's FP64 work.
template <int N>
__device__ __forceinline__ double warp_reduce_scatter(const double (&v)[N]) {
    static_assert(N >= 1 && N <= 32, "one value per lane at most");
    const int lane = threadIdx.x & 31;
    double a[32];
#pragma unroll
    for (int k = 0; k < 32; ++k) a[k] = k < N ? v[k] : 0.0;
#pragma unroll
    for (int h = 16; h >= 1; h >>= 1) {
        const bool up = (lane & h) != 0;
#pragma unroll
        for (int j = 0; j < h; ++j) {
            const double keep = up ? a[j + h] : a[j];
            const double send = up ? a[j] : a[j + h];
            a[j] = keep + __shfl_xor_sync(kPoseFull, send, h);
        }
    }
    return a[0];
}

template <class Real>
__device__ __forceinline__ void cam12(const CamState& c, Real* o) {
#pragma unroll
    for (int k = 0; k < 9; ++k) o[k] = (Real)c.R[k];
    o[9] = (Real)c.t[0];
    o[10] = (Real)c.t[1];
    o[11] = (Real)c.t[2];
}

// This thread's part of the FP64 robust chi2 of one problem at camera state c (observations
// first, first + stride, ...).
__device__ double pose_cost(const PoseArgs& A, const PoseDesc& d, const Intr& in, const CamState& c, int first,
                            int stride) {
    double cr[12];
    cam12<double>(c, cr);
    double acc = 0.0;
    for (int i = first; i < d.n; i += stride) {
        const long long k = d.o0 + i;
        const double X[3] = {A.pts[4 * k], A.pts[4 * k + 1], A.pts[4 * k + 2]};
        const double z[2] = {A.uv[2 * k], A.uv[2 * k + 1]};
        acc += edge_cost<double>(in, cr, cr + 9, X, z, A.lm.robust != 0, A.lm.huber_delta);
    }
    return acc;
}

// (H + lambda I) x = b by FP64 Cholesky of the packed lower 6x6 H; false if not positive definite.
__device__ bool chol_solve6(const double* H, double lambda, const double* b, double* x) {
    double L[21];
#pragma unroll
    for (int k = 0; k < 21; ++k) L[k] = H[k];
#pragma unroll
    for (int r = 0; r < 6; ++r) L[ptri(r, r)] += lambda;
    double rinv[6];
    bool ok = true;
#pragma unroll
    for (int j = 0; j < 6; ++j) {
        double dj = L[ptri(j, j)];
#pragma unroll
        for (int k = 0; k < j; ++k) dj -= L[ptri(j, k)] * L[ptri(j, k)];
        if (!(dj > 0.0) || !isfinite(dj)) {
            ok = false;
            dj = 1.0;
        }
        const double r = rsqrt(dj);
        rinv[j] = r;
        L[ptri(j, j)] = dj * r;
#pragma unroll
        for (int i = j + 1; i < 6; ++i) {
            double v = L[ptri(i, j)];
#pragma unroll
            for (int k = 0; k < j; ++k) v -= L[ptri(i, k)] * L[ptri(j, k)];
            L[ptri(i, j)] = v * r;
        }
    }
    double y[6];
#pragma unroll
    for (int i = 0; i < 6; ++i) {
        double s = b[i];
#pragma unroll
        for (int k = 0; k < i; ++k) s -= L[ptri(i, k)] * y[k];
        y[i] = s * rinv[i];
    }
#pragma unroll
    for (int i = 5; i >= 0; --i) {
        double s = y[i];
#pragma unroll
        for (int k = i + 1; k < 6; ++k) s -= L[ptri(k, i)] * y[k];
        y[i] = s * rinv[i];
    }
#pragma unroll
    for (int i = 0; i < 6; ++i) x[i] = ok ? y[i] : 0.0;
    return ok;
}

// One block of kPoseThreads threads per problem.  The observation passes (linearization, costs)
// stride over the block's threads; their sums go warp butterfly -> lane-parallel over the warps ->
// shared memory, in a fixed order.  Thread 0 holds the LM state and does the scalar work (6x6
// factorization, SE(3) update, gain ratio, damping), so the FP64 pipe, shared by the SM, runs it
// once; the trial state and the decisions reach the other threads through shared memory.  The
// same kernel serves every batch size, so a problem's result does not depend on its batch.
constexpr int kPoseThreads = 256;
constexpr int kPoseWarps = kPoseThreads / 32;

template <class Real>
__global__ void __launch_bounds__(kPoseThreads) pose_lm_kernel(PoseArgs A) {
    const int w = blockIdx.x;  // problem (uniform per block)
    if (w >= A.n) return;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    __shared__ double s_part[kPoseWarps][28];
    __shared__ double s_tot[28];
    __shared__ double s_hb[28];  // H (21 packed) and b (6) of the current linearization
    __shared__ CamState s_cam;  // the state the observation passes evaluate
    __shared__ int s_flag[2];
    const PoseDesc d = A.desc[w];
    const Intr in = make_intr(d.intr, d.model);
    const bool robust = A.lm.robust != 0;
    const Real delta = (Real)A.lm.huber_delta;
    // sum over the block of N per-thread values, returned in s_tot (read after the call)
    auto block_sum = [&](auto& v) {
        constexpr int nv = (int)(sizeof(v) / sizeof(v[0]));
        if constexpr (nv == 1) {
            const double t = warp_sum((double)v[0]);
            if (lane == 0) s_part[wid][0] = t;
        } else {
            double dv[nv];
#pragma unroll
            for (int k = 0; k < nv; ++k) dv[k] = (double)v[k];
            const double t = warp_reduce_scatter<nv>(dv);
            if (lane < nv) s_part[wid][lane] = t;
        }
        __syncthreads();
        if (tid < nv) {
            double t = 0.0;
#pragma unroll
            for (int i = 0; i < kPoseWarps; ++i) t += s_part[i][tid];
            s_tot[tid] = t;
        }
        __syncthreads();
    };
    auto cost_at_shared = [&]() {
        double c[1] = {pose_cost(A, d, in, s_cam, tid, kPoseThreads)};
        block_sum(c);
        return s_tot[0];
    };
    if (tid == 0) s_cam = A.cam_in[w];
    __syncthreads();
    // LM state (meaningful in thread 0; chi in every thread)
    CamState cur = s_cam, trial;
    double chi = cost_at_shared();
    const double chi0 = chi;
    int iters = 0, acc = 0, rej = 0, term = NAV_BA_TERM_ITERATIONS;
    double lambda = 0.0, nu = 2.0;
    const bool bad = !isfinite(chi);
    for (int it = 0; !bad && it < A.lm.iterations; ++it) {
        // linearize at cur (= s_cam)
        Real cr[12];
        cam12<Real>(s_cam, cr);
        Real u[27];
#pragma unroll
        for (int k = 0; k < 27; ++k) u[k] = Real(0);
        for (int i = tid; i < d.n; i += kPoseThreads) {
            const long long k = d.o0 + i;
            const Real X[3] = {(Real)A.pts[4 * k], (Real)A.pts[4 * k + 1], (Real)A.pts[4 * k + 2]};
            const Real z[2] = {(Real)A.uv[2 * k], (Real)A.uv[2 * k + 1]};
            EdgeLin<Real> L;
            edge_linearize<Real>(in, cr, cr + 9, X, z, robust, delta, L);
            const Real wt = L.w;
#pragma unroll
            for (int r = 0; r < 6; ++r)
#pragma unroll
                for (int q = 0; q <= r; ++q) u[ptri(r, q)] += wt * (L.jc[r] * L.jc[q] + L.jc[6 + r] * L.jc[6 + q]);
            const Real we0 = -wt * L.e[0], we1 = -wt * L.e[1];
#pragma unroll
            for (int r = 0; r < 6; ++r) u[21 + r] += L.jc[r] * we0 + L.jc[6 + r] * we1;
        }
        block_sum(u);
        if (tid < 27) s_hb[tid] = s_tot[tid];  // kept through the trials' cost sums
        if (tid == 0 && it == 0) {
            double mx = 0.0;
#pragma unroll
            for (int r = 0; r < 6; ++r) mx = fmax(mx, fabs(s_tot[ptri(r, r)]));
            lambda = A.lm.initial_lambda > 0 ? A.lm.initial_lambda : A.lm.tau * mx;
            nu = 2.0;
        }
        double rho = 0.0, scale = 0.0;
        int q = 0;
        for (;;) {
            // thread 0: the damped step and the trial state
            if (tid == 0) {
                double dx[6];
                const double* b = s_hb + 21;
                const bool ok = chol_solve6(s_hb, lambda, b, dx);
                se3_left_update(dx, cur, trial);
                scale = 1e-3;
#pragma unroll
                for (int r = 0; r < 6; ++r) scale += dx[r] * (lambda * dx[r] + b[r]);
                s_cam = trial;
                s_flag[0] = ok ? 1 : 0;
            }
            __syncthreads();
            const bool ok = s_flag[0] != 0;
            const double chi_new = ok ? cost_at_shared() : DBL_MAX;
            // thread 0: gain ratio and damping; whether to try again
            if (tid == 0) {
                rho = (chi - chi_new) / scale;
                if (rho > 0 && isfinite(chi_new)) {
                    double alpha = 1.0 - pow(2 * rho - 1, 3.0);
                    alpha = fmin(alpha, 2.0 / 3.0);
                    lambda *= fmax(1.0 / 3.0, alpha);
                    nu = 2.0;
                    chi = chi_new;
                    cur = trial;
                    ++acc;
                } else {
                    lambda *= nu;
                    nu *= 2;
                    ++rej;
                }
                ++q;
                s_flag[1] = (rho < 0 && q < A.lm.max_trials) ? 1 : 0;
            }
            __syncthreads();
            const bool again = s_flag[1] != 0;
            __syncthreads();  // s_flag is rewritten by the next trial
            if (!again) break;
        }
        // thread 0: termination; the next linearization point
        if (tid == 0) {
            iters = it + 1;
            int stop = 0;
            if (q == A.lm.max_trials) {
                term = NAV_BA_TERM_TRIALS_EXHAUSTED;
                stop = 1;
            } else if (rho == 0) {
                term = NAV_BA_TERM_ZERO_GAIN;
                stop = 1;
            } else if (!isfinite(lambda)) {
                term = NAV_BA_TERM_LAMBDA_NONFINITE;
                stop = 1;
            }
            s_cam = cur;
            s_flag[0] = stop;
        }
        __syncthreads();
        const bool stop = s_flag[0] != 0;
        __syncthreads();
        if (stop) break;
    }
    // observations at or behind the final pose
    __syncthreads();
    if (tid == 0) s_cam = cur;
    __syncthreads();
    double nneg[1] = {0.0};
    for (int i = tid; i < d.n; i += kPoseThreads) nneg[0] += depth_nonpositive(s_cam, A.pts + 4 * (d.o0 + i)) ? 1.0 : 0.0;
    block_sum(nneg);
    if (tid == 0) {
        A.cam_out[w] = cur;
        A.stats[w].depth_nonpos = (int32_t)s_tot[0];
        PoseStat& st = A.stats[w];
        st.initial_cost = chi0;
        st.final_cost = chi;
        st.final_lambda = lambda;
        st.iters = iters;
        st.acc = acc;
        st.rej = rej;
        st.term = term;
        st.status = bad ? NAV_BA_ERR_NONFINITE_COST : NAV_BA_OK;
    }
}

bool finite_all(const double* p, int64_t n) {
    for (int64_t i = 0; i < n; ++i)
        if (!std::isfinite(p[i])) return false;
    return true;
}

}  // namespace

void PoseBatch::release() {
    void* ps[] = {d_desc, d_cam_in, d_cam_out, d_pts, d_uv, d_stats};
    for (void* p : ps)
        if (p) cudaFree(p);
    *this = PoseBatch();
}

nav_ba_status solve_pose_batch(cudaStream_t st, PoseBatch& B, const nav_ba_pose_problem* probs, int n,
                               const nav_ba_options& o, nav_ba_pose_result* res, float* ms, std::string* why,
                               HostStaging& stg) {
    // validation of every problem on the host workers (nothing is written on error; the lowest
    // failing index is reported, as a sequential pass would)
    auto check = [&](int i, std::string* w) -> nav_ba_status {
        const nav_ba_pose_problem& p = probs[i];
        auto at = [i]() { return "pose problem " + std::to_string(i) + ": "; };
        if (p.n_obs < 0 || !p.pose || (p.n_obs > 0 && (!p.points || !p.obs_uv))) {
            *w = at() + "NULL array or negative size";
            return NAV_BA_ERR_ARGUMENT;
        }
        if (p.camera_model != NAV_BA_CAM_PINHOLE && p.camera_model != NAV_BA_CAM_PINHOLE_RADIAL &&
            p.camera_model != NAV_BA_CAM_KANNALA_BRANDT8) {
            *w = at() + "unknown camera model";
            return NAV_BA_ERR_ARGUMENT;
        }
        if (!finite_all(p.pose, 12) || !finite_all(p.intrinsics, 8) || !finite_all(p.points, 3LL * p.n_obs) ||
            !finite_all(p.obs_uv, 2LL * p.n_obs)) {
            *w = at() + "non-finite input";
            return NAV_BA_ERR_NONFINITE_INPUT;
        }
        return NAV_BA_OK;
    };
    {
        std::vector<nav_ba_status> vst(n, NAV_BA_OK);
        std::vector<std::string> vwhy(n);
        const int nth = HostPool::tasks_for(n, 16);
        stg.pool.run(nth, [&](int t) {
            for (int i = t; i < n; i += nth) vst[i] = check(i, &vwhy[i]);
        });
        for (int i = 0; i < n; ++i)
            if (vst[i] != NAV_BA_OK) {
                *why = vwhy[i];
                return vst[i];
            }
    }
    // host layout: descriptors, camera states, points [no][4], measurements [no][2]
    std::vector<PoseDesc> desc;
    std::vector<CamState> cams;
    std::vector<int32_t> slot(n, -1);
    int64_t no = 0;
    for (int i = 0; i < n; ++i) {
        if (probs[i].n_obs == 0) continue;
        slot[i] = (int32_t)desc.size();
        PoseDesc d{};
        d.o0 = no;
        d.n = probs[i].n_obs;
        d.model = probs[i].camera_model;
        for (int k = 0; k < 8; ++k) d.intr[k] = probs[i].intrinsics[k];
        desc.push_back(d);
        CamState c;
        cam_from_pose12(probs[i].pose, c);
        cams.push_back(c);
        no += probs[i].n_obs;
    }
    const int m = (int)desc.size();
    // points [no][4] and measurements [no][2] staged in pinned memory, in parallel over problems
    const size_t b_pts = sizeof(double) * 4 * std::max<int64_t>(no, 1), b_uv = sizeof(double) * 2 * std::max<int64_t>(no, 1);
    double* pts = static_cast<double*>(stg.get(0, b_pts));
    double* uv = static_cast<double*>(stg.get(1, b_uv));
    if (!pts || !uv) {
        *why = "pinned host allocation failed";
        return NAV_BA_ERR_CUDA;
    }
    {
        const int nth = HostPool::tasks_for(n, 16);
        stg.pool.run(nth, [&](int t) {
            for (int i = t; i < n; i += nth) {
                if (slot[i] < 0) continue;
                const int64_t o0 = desc[slot[i]].o0;
                const double* P = probs[i].points;
                const double* Z = probs[i].obs_uv;
                for (int64_t k = 0; k < probs[i].n_obs; ++k) {
                    double* q = pts + 4 * (o0 + k);
                    q[0] = P[3 * k];
                    q[1] = P[3 * k + 1];
                    q[2] = P[3 * k + 2];
                    q[3] = 0.0;
                }
                std::memcpy(uv + 2 * o0, Z, sizeof(double) * 2 * probs[i].n_obs);
            }
        });
    }
    std::vector<CamState> cout(std::max(1, m));
    std::vector<PoseStat> stats(std::max(1, m));
    if (m > 0) {
        cudaError_t e = cudaSuccess;
        auto ensure = [&](auto** p, size_t& cap, size_t bytes) {
            if (e != cudaSuccess) return;
            if (*p && cap >= bytes) return;
            if (*p) cudaFree(*p);
            *p = nullptr;
            cap = 0;
            e = cudaMalloc((void**)p, bytes);
            if (e == cudaSuccess) cap = bytes;
        };
        ensure(&B.d_desc, B.cap[0], sizeof(PoseDesc) * m);
        ensure(&B.d_cam_in, B.cap[1], sizeof(CamState) * m);
        ensure(&B.d_cam_out, B.cap[2], sizeof(CamState) * m);
        ensure(&B.d_pts, B.cap[3], b_pts);
        ensure(&B.d_uv, B.cap[4], b_uv);
        ensure(&B.d_stats, B.cap[5], sizeof(PoseStat) * m);
        auto upl = [&](void* d, const void* h, size_t bytes) {
            if (e == cudaSuccess) e = cudaMemcpyAsync(d, h, bytes, cudaMemcpyHostToDevice, st);
        };
        upl(B.d_desc, desc.data(), sizeof(PoseDesc) * m);
        upl(B.d_cam_in, cams.data(), sizeof(CamState) * m);
        upl(B.d_pts, pts, b_pts);
        upl(B.d_uv, uv, b_uv);
        PoseArgs A;
        A.desc = B.d_desc;
        A.n = m;
        A.cam_in = B.d_cam_in;
        A.cam_out = B.d_cam_out;
        A.pts = B.d_pts;
        A.uv = B.d_uv;
        A.stats = B.d_stats;
        LmOptions lm{};
        lm.iterations = o.iterations;
        lm.max_trials = o.max_trials;
        lm.robust = o.robust;
        lm.huber_delta = o.huber_delta;
        lm.initial_lambda = o.initial_lambda;
        lm.tau = o.tau;
        A.lm = lm;
        cudaEvent_t ev0 = nullptr, ev1 = nullptr;
        if (e == cudaSuccess) e = cudaEventCreate(&ev0);
        if (e == cudaSuccess) e = cudaEventCreate(&ev1);
        if (e == cudaSuccess) e = cudaEventRecord(ev0, st);
        if (e == cudaSuccess) {
            if (o.precision == NAV_BA_MIXED)
                pose_lm_kernel<float><<<m, kPoseThreads, 0, st>>>(A);
            else
                pose_lm_kernel<double><<<m, kPoseThreads, 0, st>>>(A);
            e = cudaGetLastError();
        }
        if (e == cudaSuccess) e = cudaEventRecord(ev1, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(cout.data(), B.d_cam_out, sizeof(CamState) * m, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(stats.data(), B.d_stats, sizeof(PoseStat) * m, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        float t = 0.f;
        if (e == cudaSuccess) cudaEventElapsedTime(&t, ev0, ev1);
        if (ev0) cudaEventDestroy(ev0);
        if (ev1) cudaEventDestroy(ev1);
        if (e != cudaSuccess) {
            *why = std::string("pose engine: ") + cudaGetErrorString(e);
            return NAV_BA_ERR_CUDA;
        }
        if (ms) *ms = t;
    }
    // a problem with a non-finite initial cost fails the call; nothing is written then
    for (int i = 0; i < n; ++i)
        if (slot[i] >= 0 && stats[slot[i]].status != NAV_BA_OK) {
            *why = "pose problem " + std::to_string(i) + ": non-finite initial cost";
            return (nav_ba_status)stats[slot[i]].status;
        }
    for (int i = 0; i < n; ++i) {
        nav_ba_pose_result& r = res[i];
        if (slot[i] < 0) {
            if (r.pose_out) std::memcpy(r.pose_out, probs[i].pose, sizeof(double) * 12);
            r.initial_cost = r.final_cost = r.final_lambda = 0.0;
            r.iterations_done = r.trials_accepted = r.trials_rejected = 0;
            r.termination = NAV_BA_TERM_NOTHING_TO_DO;
            r.status = NAV_BA_EMPTY;
            r.n_depth_nonpositive = 0;
            continue;
        }
        const PoseStat& s = stats[slot[i]];
        r.n_depth_nonpositive = s.depth_nonpos;
        r.initial_cost = s.initial_cost;
        r.final_cost = s.final_cost;
        r.final_lambda = s.final_lambda;
        r.iterations_done = s.iters;
        r.trials_accepted = s.acc;
        r.trials_rejected = s.rej;
        r.termination = s.term;
        r.status = s.status;
        if (r.pose_out) pose12_from_cam(cout[slot[i]], r.pose_out);
    }
    return NAV_BA_OK;
}

}  // namespace navba
