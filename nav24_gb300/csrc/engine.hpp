// engine.hpp - device engines behind the C ABI.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/nav_ba.h"
#include "ba_math.cuh"
#include "host_pool.hpp"
#include "structure.hpp"

namespace navba {

// Limits of the window engine (one CTA solves one window; S lives in shared memory).
constexpr int kWinMaxFreeCams = NAV_BA_WINDOW_MAX_CAMS;  // 6*24 = 144 reduced unknowns
constexpr int kWinMaxCams = 64;                          // cameras per window, fixed ones included

struct WinDesc {
    int32_t cam0, ncam;   // camera range (global)
    int32_t pt0, npt;     // point range (global)
    int32_t e0, ne;       // active-edge range (global), point-major
    int32_t nfc, nfp;     // free cameras / points
    int64_t pair0;        // first slot of the window's Schur pair list (global)
    int64_t npair;        // pair-list length
    int64_t s0;           // mixed form: first value of the window's FP64 reduced system (global scratch)
};

struct WinStats {
    double initial_cost, final_cost, final_lambda;
    int32_t iterations_done, accepted, rejected, termination;
    int32_t status;
    int32_t depth_nonpos;  // active edges with the point at or behind its camera, final state
    int32_t pad1, pad2;
};

// Per-launch options of the LM loop.
struct LmOptions {
    int32_t iterations;
    int32_t max_trials;
    int32_t robust;
    int32_t solver;          // NAV_BA_SOLVER_CHOLESKY / NAV_BA_SOLVER_PCG
    double huber_delta;
    double initial_lambda;
    double tau;
    int32_t optimize_k;      // shared radial k1, k2 are free (PCG only)
    int32_t pcg_max_iterations;
    double pcg_tolerance;
};

// A batch of windows resident on the device (inputs, scratch and outputs).
struct WindowBatch {
    int32_t n_win = 0;        // windows in the batch (stats/trace rows)
    int32_t n_queue = 0;      // windows the kernel solves (the work queue)
    int64_t ncam = 0, npt = 0, ne = 0, npair = 0;
    int32_t max_m = 0;        // largest 6 * nfc in the batch
    int32_t max_ncam = 0;     // largest camera count in the batch
    int32_t precision = 0;    // buffers sized for this precision
    int32_t trace_stride = 0; // iterations + 1
    // device inputs
    WinDesc* d_win = nullptr;
    int32_t* d_order = nullptr;
    int32_t* d_queue = nullptr;
    CamState* d_cam_init = nullptr;
    int32_t* d_cam_free = nullptr;
    double* d_pt_init = nullptr;   // [npt][4]
    int32_t* d_pt_free = nullptr;
    int32_t* d_pt_eoff = nullptr;  // [npt + 1] global edge offsets
    int32_t* d_edge_cam = nullptr; // window-local camera of each edge
    int32_t* d_edge_fc = nullptr;  // free index of each edge's camera, or -1
    int32_t* d_edge_pt = nullptr;  // window-local point of each edge
    double* d_edge_uv = nullptr;   // [ne][2]
    // device scratch
    double* d_x[2] = {nullptr, nullptr};  // [npt][4] current / trial points
    void* d_pt_vg = nullptr;       // [npt][12] Real: V (6 packed) g (3)
    void* d_pt_lt = nullptr;       // [npt][12] Real: Linv (6 packed lower) t = Linv g (3)
    void* d_edge_w = nullptr;      // FP64 form: [ne][18] W = w Jc^T Jp (the mixed form recomputes W)
    void* d_edge_a = nullptr;      // [ne][20 f32 | 18 f64] Real: A = W Linv^T
    void* d_edge_e[2] = {nullptr, nullptr};  // mixed: [ne][2] f32 residuals, current / trial state
    int32_t* d_cam_list = nullptr; // [ne] camera-major edge list (free cameras only)
    uint32_t* d_pairs = nullptr;   // [npair] Schur pairs (edge i << 16 | edge j), window-local
    void* d_edge_uvr = nullptr;    // mixed: [ne][2] f32 observations
    double* d_s = nullptr;         // mixed: the windows' packed FP64 reduced systems (sum of m(m+1)/2)
    void* d_xr[2] = {nullptr, nullptr};  // mixed: [npt][4] f32 copies of d_x
    // device outputs
    CamState* d_cam_out = nullptr;
    double* d_pt_out = nullptr;    // [npt][4]
    double* d_trace = nullptr;     // [n_win][trace_stride]
    WinStats* d_stats = nullptr;
    double* d_debug = nullptr;     // reduced-system debug output (optional)
    unsigned long long* d_phase = nullptr;  // per-phase cycle totals (NAVBA_PHASE_TIMING=1)
    std::vector<double> order_weight;  // host: work weight of each window in queue order (decreasing)
    size_t cap[48] = {};      // allocated bytes of each buffer (buffers are reused across calls)
    size_t bytes = 0;
    int64_t h2d_bytes = 0;    // bytes uploaded by window_batch_upload
};

// Launch shape of the window kernel (picked by the autotuner).  With cluster > 1, the windows whose
// work weight (WindowBatch::order_weight) is at least big_weight are each solved by a whole cluster
// and the others by single CTAs; big_weight 0: every window by a cluster.
struct WindowLaunch {
    int32_t cluster = 4;      // CTAs cooperating on one large window (1, 2, 4 or 8)
    int32_t threads = 256;    // threads per CTA
    double big_weight = 0.0;
};

// Host resources of a context reused across calls: pinned buffers (inputs staged for upload,
// outputs for download) and the worker threads of the host-side passes.
struct HostStaging {
    void* buf[16] = {};
    size_t cap[16] = {};
    HostPool pool;
    void* get(int id, size_t bytes);  // grows buffer `id` to at least `bytes`; null on failure
    void release();
};

// Host side of a prepared batch: the built windows and their device copy.
struct PreparedBatch {
    std::vector<HostWindow> host;
    std::vector<int32_t> host_status;  // per window: NAV_BA_OK / NAV_BA_EMPTY / error
    std::vector<WinDesc> desc;
    WindowBatch dev;
    LmOptions lm{};
    Intr intr{};
};

// Allocate (reusing pb.dev's buffers when large enough) and upload through pinned staging.
// Synchronous on return unless sync is false: then the copies are in flight on `stream`, and stg
// must not be restaged before the stream has passed them.  Returns a CUDA error or 0.
cudaError_t window_batch_upload(PreparedBatch& pb, cudaStream_t stream, int precision,
                                int trace_stride, HostStaging& stg, HostPool& pool, std::string* why,
                                bool sync = true);
void window_batch_free(WindowBatch& b);

// Launch the persistent window kernel over all windows of the batch.
// debug_lambda >= 0 stops after assembling the reduced system of window 0 at that damping
// and writes [S (m*m) | b (m)] to d_debug.
cudaError_t window_batch_launch(PreparedBatch& pb, cudaStream_t stream, int precision,
                                WindowLaunch shape, double debug_lambda);

// Print the per-phase cycle breakdown of the last launch to stderr (NAVBA_PHASE_TIMING=1).
constexpr int kWinPhases = 16;
struct WindowLaunch;
void window_phase_report(const PreparedBatch& pb, const WindowLaunch& shape, int precision);

// Shared memory one CTA of the window kernel needs for a batch (bytes).
size_t window_smem_bytes(int max_m, int max_ncam, int precision);

// Linearize every observation of a problem at its initial state (device, precision given);
// outputs in observation order, FP64.
cudaError_t linearize_observations(const nav_ba_problem& p, const nav_ba_options& o,
                                   cudaStream_t stream, double* e, double* jc, double* jp,
                                   double* w, std::string* why);

// Result of one grid-engine solve (grid_engine.cu).
struct GridResult {
    int32_t status = 0;
    double initial_cost = 0, final_cost = 0, final_lambda = 0;
    int32_t iterations_done = 0, accepted = 0, rejected = 0, termination = 0;
    std::vector<double> trace;
    std::vector<CamState> cams;
    std::vector<double> points;  // [npt][4]
    double k1 = 0, k2 = 0;       // final distortion (optimize_k)
    int32_t pcg_iterations = 0;
    int32_t depth_nonpos = 0;    // active edges with the point at or behind its camera, final state
};

// Differentiation through the accepted LM steps (grid engine, FP64, Cholesky, pinhole).
struct GridVjp {
    // replay: apply the steps of `lambdas` unconditionally; else run LM and record the damping of
    // every accepted step into `lambdas`
    bool replay = false;
    std::vector<double> lambdas;
    // backward: run it with these cotangents of the outputs (problem order; null = zero)
    bool backward = false;
    double cost_bar = 0.0;
    const double* pose_bar = nullptr;   // [ncam][12]
    const double* point_bar = nullptr;  // [npt][3]
    // results of the backward
    std::vector<double> uv_bar;         // [ne][2], active-edge order
    double intr_bar[4] = {0, 0, 0, 0};  // fx, fy, cx, cy
    std::vector<double> cam_bar;        // [ncam][6] left-tangent adjoint of the input poses
    std::vector<double> pt_bar;         // [npt][3]
    std::string why;                    // reason of a non-OK status
};

struct GridWorkspace;

// Solve one large problem on the whole GPU.  debug_S != nullptr: stop after assembling the
// reduced system at damping debug_lambda and return [S (m*m, row-major, lower part) | b'].
// vjp != nullptr (FP64 only): record or replay the damping schedule and run the backward.
// ws: buffers kept across calls (nullptr: the call allocates and frees its own, pageable read-backs).
cudaError_t grid_solve(const HostWindow& h, const LmOptions& lm, const Intr& intr, int precision,
                       cudaStream_t stream, HostPool* pool, GridWorkspace* ws, GridResult& out,
                       double debug_lambda, std::vector<double>* debug_S, GridVjp* vjp = nullptr);

// Motion-only BA (pose_engine.cu): per problem descriptor, statistics, and the reused device buffers.
struct PoseDesc {
    int64_t o0;       // first observation (global)
    int32_t n;        // observations
    int32_t model;    // camera model
    double intr[8];   // fx fy cx cy k1 k2 k3 k4
};
struct PoseStat {
    double initial_cost, final_cost, final_lambda;
    int32_t iters, acc, rej, term, status;
    int32_t depth_nonpos;  // observations at or behind the final pose
};
struct PoseBatch {
    PoseDesc* d_desc = nullptr;
    CamState* d_cam_in = nullptr;
    CamState* d_cam_out = nullptr;
    double* d_pts = nullptr;   // [no][4]
    double* d_uv = nullptr;    // [no][2]
    PoseStat* d_stats = nullptr;
    size_t cap[6] = {};
    void release();
};
// stg: pinned staging and host workers (the call is synchronous on return)
nav_ba_status solve_pose_batch(cudaStream_t stream, PoseBatch& B, const nav_ba_pose_problem* probs, int n,
                               const nav_ba_options& o, nav_ba_pose_result* res, float* ms, std::string* why,
                               HostStaging& stg);

// Two-view triangulation and hypothesis checks (twoview.cu).
// Grow-only device scratch of a context for its synchronous small calls (two-view check,
// undistortion): no allocation, and no free (which synchronizes the device), per call.
struct DevScratch {
    void* p = nullptr;
    size_t cap = 0;
    void* get(size_t bytes, cudaError_t* e) {
        if (p && cap >= bytes) return p;
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
        *e = cudaMalloc(&p, std::max<size_t>(bytes, 256));
        if (*e != cudaSuccess) {
            p = nullptr;
            return nullptr;
        }
        cap = std::max<size_t>(bytes, 256);
        return p;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
    }
};

// Buffers of grid-engine solves kept by a context across calls (one context per host thread).
// - slab: device memory the next call carves its buffers from, grown at the end of a call to what
//   that call needed (the largest so far); a call that finds the slab too small allocates the
//   rest buffer by buffer.
// - pinned: page-locked host memory for the per-trial read-backs, grown on demand.
// A call holds the workspace while it runs (busy); a call that finds it held works without it.
// NAVBA_GRID_WORKSPACE=0 turns the slab off (every call allocates and frees its own buffers).
struct GridWorkspace {
    DevScratch slab;
    bool busy = false;
    void* pinned = nullptr;
    size_t pinned_cap = 0;
    void release() {
        slab.release();
        if (pinned) cudaFreeHost(pinned);
        pinned = nullptr;
        pinned_cap = 0;
    }
};

nav_ba_status twoview_check(cudaStream_t stream, const nav_ba_twoview& in, nav_ba_twoview_result& out, std::string* why,
                            DevScratch& scratch);

// Keypoint undistortion (undistort.cu).
nav_ba_status undistort_points(cudaStream_t stream, const double* K, const double* dist, int iters, int n,
                               const double* uv_in, double* uv_out, std::string* why, DevScratch& scratch);

// One-window solve in the library's static device array (no device allocation), noalloc.cu.
nav_ba_status solve_window_noalloc(int device, cudaStream_t stream, const nav_ba_problem& p,
                                   const nav_ba_options& o, nav_ba_result& r, std::string* why);

}  // namespace navba
