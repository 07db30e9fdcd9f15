// nav_ba_api.cu - the C ABI of include/nav_ba.h.
//
// Replaces nav24's GraphOptim::solve (core/backEnd/BE_GraphOptim.cpp:31-77): graph build
// (structure.cpp), LM on the device (window_engine.cu), write-back of poses and points.
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "engine.hpp"

using namespace navba;

// Parts of a pipelined batched solve (8 measured slower: 64-window parts leave host workers idle).
constexpr int kSolveParts = 4;
static_assert(kSolveParts == 4, "NAVBA_PART_BOUNDS parses three inner boundaries");
// The shape of the first part of a pipelined batch (the largest windows), by precision
// (NAV_BA_FP64, NAV_BA_MIXED): clusters over a window of that part, measured best on the
// 256-window workload (FP64 4 x 128 threads, mixed 2 x 256; 1 to 8 CTAs lie within 1 to 10 %).
constexpr WindowLaunch kPart0Shape[2] = {{4, 128, 0.0}, {2, 256, 0.0}};

struct nav_ba_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    std::string last_error;
    PreparedBatch prepared;
    std::vector<nav_ba_problem> prepared_problems;  // shapes of the prepared problem (no data)
    nav_ba_options prepared_opts{};
    PoseBatch pose;  // device buffers of nav_ba_solve_pose_batched (reused)
    DevScratch scratch;  // device buffer of the two-view check and the undistortion (reused)
    bool has_prepared = false;
    WindowLaunch shape[2];        // per precision (autotuned on nav_ba_prepare_batched)
    bool tuned[2] = {false, false};
    WindowBatch solve_dev;        // device buffers of nav_ba_solve / _batched, reused across calls
    std::vector<HostWindow> solve_host;  // their host-side windows, reused across calls
    HostStaging stg;              // pinned staging reused across calls
    GridWorkspace gws;            // device and pinned buffers of grid-engine solves, reused across calls
    // pipelined batched solves: the batch's parts, each with its windows, device buffers, pinned
    // staging and stream (the host builds part k + 1 while the device solves part k)
    struct Part {
        std::vector<HostWindow> host;
        WindowBatch dev;
        HostStaging stg;
        cudaStream_t stream = nullptr;
    };
    Part parts[kSolveParts];
    // nav_ba_run's launch sequence over the prepared batch (queue reset, persistent kernel),
    // captured once in a CUDA graph at prepare time and replayed by every run with the same options
    cudaGraphExec_t run_graph = nullptr;
    LmOptions graph_lm{};
};

namespace {

double ms_since(std::chrono::steady_clock::time_point t0) {
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

nav_ba_status set_err(nav_ba_ctx* ctx, nav_ba_status st, const std::string& msg) {
    if (ctx) ctx->last_error = msg;
    return st;
}

nav_ba_status cuda_status(nav_ba_ctx* ctx, cudaError_t e, const char* where) {
    if (e == cudaSuccess) return NAV_BA_OK;
    const nav_ba_status st = (e == cudaErrorMemoryAllocation) ? NAV_BA_ERR_OUT_OF_MEMORY : NAV_BA_ERR_CUDA;
    return set_err(ctx, st, std::string(where) + ": " + cudaGetErrorString(e));
}

LmOptions lm_options(const nav_ba_options& o) {
    LmOptions lm{};
    lm.iterations = o.iterations;
    lm.max_trials = o.max_trials;
    lm.robust = o.robust;
    lm.huber_delta = o.huber_delta;
    lm.initial_lambda = o.initial_lambda;
    lm.tau = o.tau;
    lm.solver = o.solver;
    lm.optimize_k = o.optimize_distortion;
    lm.pcg_max_iterations = o.pcg_max_iterations;
    lm.pcg_tolerance = o.pcg_tolerance;
    return lm;
}

Intr intrinsics_of(const nav_ba_problem& p) {
    return make_intr(p.intrinsics, p.camera_model);
}

// Outputs of a problem nothing is done to: the round-trip of each pose through its quaternion
// (as nav24's recoverPose writes every pose vertex back) and the input points.
void write_passthrough(const nav_ba_problem& p, nav_ba_result* r, bool roundtrip) {
    if (r->cam_pose_out) {
        for (int c = 0; c < p.n_cams; ++c) {
            if (roundtrip) {
                CamState cs;
                cam_from_pose12(p.cam_pose + 12LL * c, cs);
                pose12_from_cam(cs, r->cam_pose_out + 12LL * c);
            } else {
                std::memcpy(r->cam_pose_out + 12LL * c, p.cam_pose + 12LL * c, sizeof(double) * 12);
            }
        }
    }
    if (r->points_out) std::memcpy(r->points_out, p.points, sizeof(double) * 3 * p.n_points);
    if (r->intrinsics_out) std::memcpy(r->intrinsics_out, p.intrinsics, sizeof(double) * 8);
}

void clear_stats(nav_ba_result* r) {
    r->initial_cost = r->final_cost = r->final_lambda = 0.0;
    r->time_setup_ms = r->time_solve_ms = r->time_download_ms = 0.0;
    r->iterations_done = r->trials_accepted = r->trials_rejected = 0;
    r->termination = NAV_BA_TERM_ITERATIONS;
    r->n_active_edges = r->n_free_cams = r->n_free_points = r->n_schur_blocks = 0;
    r->pcg_iterations_total = 0;
    r->status = NAV_BA_OK;
    r->edge_iterations = r->h2d_bytes = r->d2h_bytes = 0;
    r->n_depth_nonpositive = 0;
}

// host_status of a window that goes to the grid engine (too large for the window engine)
constexpr int32_t kGridWindow = 2;

bool fits_window_engine(const HostWindow& h) {
    return h.nfc <= kWinMaxFreeCams && h.ncam <= kWinMaxCams && h.ne < 65536;
}

// Autotuner of the window kernel's launch shape and per-window schedule: every candidate (cluster
// size x threads per CTA x which windows the clusters solve) solves the prepared batch twice; the
// fastest is kept for the context and precision.  The windows a cluster solves are those whose work
// weight is at least a quantile of the batch's weights (the top 1, 3, 10, 25 or 100%); the others
// are solved by single CTAs.  NAVBA_WINDOW_SHAPE="<cluster>,<threads>[,<big_weight>]" fixes the
// shape instead (no tuning launches), e.g. to profile one known launch.
cudaError_t autotune(nav_ba_ctx* ctx, PreparedBatch& pb, int precision) {
    const char* fixed = getenv("NAVBA_WINDOW_SHAPE");
    int fc = 0, ft = 0;
    double fw = 0.0;
    if (fixed && sscanf(fixed, "%d,%d,%lf", &fc, &ft, &fw) >= 2 && (fc == 1 || fc == 2 || fc == 4 || fc == 8) &&
        (ft == 128 || ft == 256 || (ft == 512 && precision == NAV_BA_MIXED))) {
        ctx->shape[precision] = WindowLaunch{fc, ft, fw};
        ctx->tuned[precision] = true;
        return cudaSuccess;
    }
    // 128-thread CTAs put more windows in flight per SM (the same registers per thread)
    const int ths_fp64[] = {128, 256};
    const int ths_mixed[] = {128, 256, 512};
    const int* ths = precision == NAV_BA_MIXED ? ths_mixed : ths_fp64;
    const int nth = precision == NAV_BA_MIXED ? 3 : 2;
    const int clusters[] = {1, 2, 4, 8};
    // weight thresholds: the order weights are decreasing, so the top fraction f starts at index f n
    const std::vector<double>& ow = pb.dev.order_weight;
    std::vector<double> cuts;
    for (const double f : {0.01, 0.03, 0.10, 0.25}) {
        if (ow.empty()) break;
        const size_t k = std::min(ow.size() - 1, (size_t)std::ceil(f * (double)ow.size()) - 1);
        cuts.push_back(ow[k]);
    }
    cuts.push_back(0.0);  // every window by a cluster
    float best = 1e30f;
    WindowLaunch best_shape = ctx->shape[precision];
    std::vector<WindowLaunch> cands;
    for (int ci = 0; ci < 4; ++ci)
        for (int ti = 0; ti < nth; ++ti) {
            if (clusters[ci] == 1) {
                cands.push_back(WindowLaunch{1, ths[ti], 0.0});
                continue;
            }
            for (const double w : cuts) cands.push_back(WindowLaunch{clusters[ci], ths[ti], w});
        }
    for (const WindowLaunch& sh : cands) {
        // the shape's time is the better of two launches (the first may run on a cold L2)
        float t = 1e30f;
        bool skip = false;
        for (int rep = 0; rep < 2 && !skip; ++rep) {
            cudaEventRecord(ctx->ev0, ctx->stream);
            cudaError_t e = window_batch_launch(pb, ctx->stream, precision, sh, -1.0);
            cudaEventRecord(ctx->ev1, ctx->stream);
            if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
            if (e != cudaSuccess) {
                // a shape that cannot launch (occupancy) is skipped; any other error is reported
                if (e == cudaErrorInvalidConfiguration || e == cudaErrorInvalidValue) {
                    cudaGetLastError();
                    skip = true;
                    continue;
                }
                return e;
            }
            float tr = 0.f;
            cudaEventElapsedTime(&tr, ctx->ev0, ctx->ev1);
            t = std::min(t, tr);
        }
        if (skip) continue;
        if (t < best) {
            best = t;
            best_shape = sh;
        }
    }
    ctx->shape[precision] = best_shape;
    ctx->tuned[precision] = true;
    const char* env = getenv("NAVBA_VERBOSE");
    if (env && env[0] == '1')
        fprintf(stderr, "[navba autotune] precision=%d cluster=%d threads=%d big_weight=%.0f %.3f ms\n", precision,
                best_shape.cluster, best_shape.threads, best_shape.big_weight, best);
    return cudaSuccess;
}

// Captures the prepared batch's launch sequence in ctx->run_graph (null if capture fails: the runs
// then launch directly).
void capture_run_graph(nav_ba_ctx* ctx, int precision) {
    if (ctx->run_graph) cudaGraphExecDestroy(ctx->run_graph);
    ctx->run_graph = nullptr;
    cudaGraph_t g = nullptr;
    if (cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeRelaxed) != cudaSuccess) {
        cudaGetLastError();
        return;
    }
    const cudaError_t le = window_batch_launch(ctx->prepared, ctx->stream, precision, ctx->shape[precision], -1.0);
    cudaError_t e = cudaStreamEndCapture(ctx->stream, &g);
    if (le == cudaSuccess && e == cudaSuccess && g) e = cudaGraphInstantiate(&ctx->run_graph, g, 0);
    if (g) cudaGraphDestroy(g);
    if (le != cudaSuccess || e != cudaSuccess) {
        if (ctx->run_graph) cudaGraphExecDestroy(ctx->run_graph);
        ctx->run_graph = nullptr;
        cudaGetLastError();
        return;
    }
    ctx->graph_lm = ctx->prepared.lm;
}

// Checks of problem i of a batch: validate_problem and the batch rules (one calibration, one camera
// model, distortion optimization only with PCG).
nav_ba_status check_problem(const nav_ba_problem* probs, int i, const nav_ba_options* o, std::string* why) {
    nav_ba_status s = validate_problem(&probs[i], why);
    if (s == NAV_BA_OK && o->optimize_distortion && probs[i].camera_model == NAV_BA_CAM_PINHOLE_RADIAL &&
        o->solver != NAV_BA_SOLVER_PCG) {
        s = NAV_BA_ERR_UNSUPPORTED;
        *why = "distortion optimization needs the PCG solver";
    }
    if (s == NAV_BA_OK && i > 0 && std::memcmp(probs[i].intrinsics, probs[0].intrinsics, sizeof(double) * 8) != 0) {
        s = NAV_BA_ERR_UNSUPPORTED;
        *why = "a batch shares one calibration";
    }
    if (s == NAV_BA_OK && i > 0 && probs[i].camera_model != probs[0].camera_model) {
        s = NAV_BA_ERR_UNSUPPORTED;
        *why = "a batch shares one camera model";
    }
    return s;
}

// The options and every problem of a batch checked over the host workers; the first failing
// problem (lowest index) is reported, as a sequential pass would.
nav_ba_status check_batch(nav_ba_ctx* ctx, const nav_ba_problem* probs, int n, const nav_ba_options* o) {
    std::string why;
    nav_ba_status st = validate_options(o, &why);
    if (st != NAV_BA_OK) return set_err(ctx, st, why);
    if (o->solver == NAV_BA_SOLVER_PCG && o->pcg_max_iterations < 1)
        return set_err(ctx, NAV_BA_ERR_ARGUMENT, "pcg_max_iterations < 1");
    std::vector<nav_ba_status> vst(n, NAV_BA_OK);
    std::vector<std::string> vwhy(n);
    const int nth = HostPool::tasks_for(n, 8);
    ctx->stg.pool.run(nth, [&](int t) {
        for (int i = t; i < n; i += nth) vst[i] = check_problem(probs, i, o, &vwhy[i]);
    });
    for (int i = 0; i < n; ++i)
        if (vst[i] != NAV_BA_OK) return set_err(ctx, vst[i], "problem " + std::to_string(i) + ": " + vwhy[i]);
    return NAV_BA_OK;
}

// Validate and build all windows on the host.  Returns an error (nothing written) or OK.
// checked: the caller has run check_batch over these problems already.
nav_ba_status build_batch(nav_ba_ctx* ctx, const nav_ba_problem* probs, int n, const nav_ba_options* o,
                          PreparedBatch& pb, bool checked = false) {
    std::string why;
    nav_ba_status st = validate_options(o, &why);
    if (st != NAV_BA_OK) return set_err(ctx, st, why);
    if (o->solver == NAV_BA_SOLVER_PCG && o->pcg_max_iterations < 1)
        return set_err(ctx, NAV_BA_ERR_ARGUMENT, "pcg_max_iterations < 1");
    // validation and graph build of every problem spread over host threads; the first failing
    // problem (lowest index) is reported, as a sequential pass would
    pb.host.resize(n);  // the windows' host arrays are reused across calls (build_window rewrites them)
    pb.host_status.assign(n, NAV_BA_OK);
    std::vector<nav_ba_status> vst(n, NAV_BA_OK);
    std::vector<std::string> vwhy(n);
    const int nth = HostPool::tasks_for(n, 2);
    auto work = [&](int t) {
        for (int i = t; i < n; i += nth) {
            const nav_ba_status s = checked ? NAV_BA_OK : check_problem(probs, i, o, &vwhy[i]);
            vst[i] = s;
            if (s != NAV_BA_OK) continue;
            build_window(probs[i], *o, pb.host[i]);
            const HostWindow& h = pb.host[i];
            if (probs[i].n_cams == 0 || h.ne == 0) pb.host_status[i] = NAV_BA_EMPTY;
        }
    };
    ctx->stg.pool.run(nth, work);
    for (int i = 0; i < n; ++i)
        if (vst[i] != NAV_BA_OK)
            return set_err(ctx, vst[i], "problem " + std::to_string(i) + ": " + vwhy[i]);
    for (int i = 0; i < n; ++i)
        if (pb.host_status[i] == NAV_BA_OK && (o->solver == NAV_BA_SOLVER_PCG || !fits_window_engine(pb.host[i])))
            pb.host_status[i] = kGridWindow;  // the window engine is Cholesky-only
    pb.lm = lm_options(*o);
    pb.intr = n > 0 ? intrinsics_of(probs[0]) : Intr{};
    return NAV_BA_OK;
}

// Download results of every window into results[] (outputs of EMPTY windows: passthrough).
nav_ba_status download_batch(nav_ba_ctx* ctx, const nav_ba_problem* probs, int n, PreparedBatch& pb,
                             nav_ba_result* results, HostStaging* stg_in = nullptr, cudaStream_t stream = nullptr) {
    WindowBatch& b = pb.dev;
    HostStaging& stg = stg_in ? *stg_in : ctx->stg;
    if (!stg_in) stream = ctx->stream;
    CamState* cams = (CamState*)stg.get(10, sizeof(CamState) * b.ncam);
    double* pts = (double*)stg.get(11, sizeof(double) * 4 * b.npt);
    double* trace = (double*)stg.get(12, sizeof(double) * (size_t)b.trace_stride * n);
    WinStats* stats = (WinStats*)stg.get(13, sizeof(WinStats) * n);
    if (!cams || !pts || !trace || !stats) return set_err(ctx, NAV_BA_ERR_OUT_OF_MEMORY, "pinned host allocation failed");
    cudaError_t e = cudaSuccess;
    int64_t d2h = 0;
    auto dn = [&](void* dst, const void* src, size_t bytes) {
        if (e != cudaSuccess || bytes == 0) return;
        e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, stream);
        d2h += (int64_t)bytes;
    };
    dn(cams, b.d_cam_out, sizeof(CamState) * b.ncam);
    dn(pts, b.d_pt_out, sizeof(double) * 4 * b.npt);
    dn(trace, b.d_trace, sizeof(double) * (size_t)b.trace_stride * n);
    dn(stats, b.d_stats, sizeof(WinStats) * n);
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    if (e != cudaSuccess) return cuda_status(ctx, e, "download");
    std::vector<int32_t> st_out(n, NAV_BA_OK);
    auto one = [&](int i) {
        nav_ba_result* r = &results[i];
        const nav_ba_problem& p = probs[i];
        const HostWindow& h = pb.host[i];
        const WinDesc& d = pb.desc[i];
        r->n_active_edges = h.ne;
        r->n_free_cams = h.nfc;
        r->n_free_points = h.nfp;
        r->n_schur_blocks = h.n_schur_blocks;
        r->h2d_bytes = b.h2d_bytes;
        r->d2h_bytes = d2h;
        if (pb.host_status[i] == NAV_BA_EMPTY) {
            write_passthrough(p, r, false);
            r->termination = NAV_BA_TERM_NOTHING_TO_DO;
            r->status = NAV_BA_EMPTY;
            return;
        }
        if (pb.host_status[i] == kGridWindow) return;  // solved by the grid engine
        const WinStats& s = stats[i];
        r->status = s.status;
        r->initial_cost = s.initial_cost;
        r->final_cost = s.final_cost;
        r->final_lambda = s.final_lambda;
        r->iterations_done = s.iterations_done;
        r->trials_accepted = s.accepted;
        r->trials_rejected = s.rejected;
        r->termination = s.termination;
        r->edge_iterations = (int64_t)h.ne * s.iterations_done;
        r->n_depth_nonpositive = s.depth_nonpos;
        if (s.status != NAV_BA_OK) {
            st_out[i] = s.status;
            return;
        }
        if (r->cam_pose_out)
            for (int c = 0; c < p.n_cams; ++c) pose12_from_cam(cams[d.cam0 + c], r->cam_pose_out + 12LL * c);
        if (r->points_out)
            for (int k = 0; k < p.n_points; ++k)
                for (int j = 0; j < 3; ++j) r->points_out[3LL * k + j] = pts[4LL * (d.pt0 + k) + j];
        if (r->intrinsics_out) std::memcpy(r->intrinsics_out, p.intrinsics, sizeof(double) * 8);
        if (r->cost_trace)
            for (int k = 0; k <= s.iterations_done; ++k) r->cost_trace[k] = trace[(size_t)i * b.trace_stride + k];
    };
    const int nth = HostPool::tasks_for(n, 8);
    ctx->stg.pool.run(nth, [&](int t) {
        for (int i = (int)((long long)n * t / nth); i < (int)((long long)n * (t + 1) / nth); ++i) one(i);
    });
    for (int i = 0; i < n; ++i)
        if (st_out[i] != NAV_BA_OK) return (nav_ba_status)st_out[i];
    return NAV_BA_OK;
}

// Outputs and statistics of a grid-engine solve.
void fill_grid_result(const nav_ba_problem& p, const HostWindow& h, const nav_ba_options& o, const GridResult& g,
                      nav_ba_result& r) {
    r.status = NAV_BA_OK;
    r.initial_cost = g.initial_cost;
    r.final_cost = g.final_cost;
    r.final_lambda = g.final_lambda;
    r.iterations_done = g.iterations_done;
    r.trials_accepted = g.accepted;
    r.trials_rejected = g.rejected;
    r.termination = g.termination;
    r.n_active_edges = h.ne;
    r.n_free_cams = h.nfc;
    r.n_free_points = h.nfp;
    r.n_schur_blocks = h.n_schur_blocks;
    r.edge_iterations = (int64_t)h.ne * g.iterations_done;
    r.n_depth_nonpositive = g.depth_nonpos;
    if (r.cam_pose_out)
        for (int c = 0; c < p.n_cams; ++c) pose12_from_cam(g.cams[c], r.cam_pose_out + 12LL * c);
    if (r.points_out)
        for (int k = 0; k < p.n_points; ++k)
            for (int j = 0; j < 3; ++j) r.points_out[3LL * k + j] = g.points[4LL * k + j];
    if (r.intrinsics_out) {
        std::memcpy(r.intrinsics_out, p.intrinsics, sizeof(double) * 8);
        if (o.optimize_distortion && p.camera_model == NAV_BA_CAM_PINHOLE_RADIAL) {
            r.intrinsics_out[4] = g.k1;
            r.intrinsics_out[5] = g.k2;
        }
    }
    r.pcg_iterations_total = g.pcg_iterations;
    if (r.cost_trace)
        for (int k = 0; k <= g.iterations_done; ++k) r.cost_trace[k] = g.trace[k];
}

// One problem beyond the window engine's limits, on the grid engine; fills r (outputs and stats).
nav_ba_status solve_grid_window(nav_ba_ctx* ctx, const nav_ba_problem& p, const HostWindow& h, const nav_ba_options& o,
                                nav_ba_result& r) {
    GridResult g;
    cudaEventRecord(ctx->ev0, ctx->stream);
    cudaError_t e = grid_solve(h, lm_options(o), intrinsics_of(p), o.precision, ctx->stream, &ctx->stg.pool, &ctx->gws,
                               g, -1.0, nullptr);
    cudaEventRecord(ctx->ev1, ctx->stream);
    if (e == cudaSuccess) e = cudaEventSynchronize(ctx->ev1);
    if (e != cudaSuccess) return cuda_status(ctx, e, "grid engine");
    if (g.status != NAV_BA_OK) return set_err(ctx, (nav_ba_status)g.status, "non-finite initial cost");
    float t = 0.f;
    cudaEventElapsedTime(&t, ctx->ev0, ctx->ev1);
    fill_grid_result(p, h, o, g, r);
    r.time_solve_ms += t;
    return NAV_BA_OK;
}

// Batched solve in parts pipelined across the host and the device: part k is built on the host,
// staged and uploaded, and its window kernel launched on the part's stream; the host goes on with
// part k + 1 while the device solves part k (the parts' kernels also run side by side).  A window
// is solved start to finish by one cluster (several milliseconds for the largest), so the parts take
// the windows largest first: the first part's windows set the critical path and go to the device
// as early as possible; the last part, launched last, holds the smallest windows.  Windows are independent, so the results equal those of one launch over
// the batch.  Each part's build checks its problems; on a failure the whole batch is checked in
// the caller's order, so errors are reported as by the single-launch path (the first failing
// problem, nothing written).
constexpr int kPipelineMinWindows = 64;

nav_ba_status solve_pipelined(nav_ba_ctx* ctx, const nav_ba_problem* probs, int n, const nav_ba_options* o,
                              nav_ba_result* results) {
    const auto t0 = std::chrono::steady_clock::now();
    // the options here; each problem is checked by its part's build, so the device starts on the
    // first part before the rest of the batch is checked.  A failure is reported by one check over
    // the caller's order (the lowest failing index, as a single pass would), after the parts already
    // launched have finished; nothing is written to the results.
    nav_ba_status st = NAV_BA_OK;
    {
        std::string why;
        st = validate_options(o, &why);
        if (st != NAV_BA_OK) return set_err(ctx, st, why);
        if (o->solver == NAV_BA_SOLVER_PCG && o->pcg_max_iterations < 1)
            return set_err(ctx, NAV_BA_ERR_ARGUMENT, "pcg_max_iterations < 1");
    }
    // windows by decreasing size (observations, then cameras); part k takes the k-th quarter
    std::vector<int32_t> perm(n);
    for (int i = 0; i < n; ++i) perm[i] = i;
    std::stable_sort(perm.begin(), perm.end(), [&](int32_t x, int32_t y) {
        if (probs[x].n_obs != probs[y].n_obs) return probs[x].n_obs > probs[y].n_obs;
        return probs[x].n_cams > probs[y].n_cams;
    });
    std::vector<nav_ba_problem> pp(n);
    for (int j = 0; j < n; ++j) pp[j] = probs[perm[j]];
    PreparedBatch pbs[kSolveParts];
    for (int k = 0; k < kSolveParts; ++k) {
        auto& part = ctx->parts[k];
        if (!part.stream && cudaStreamCreateWithFlags(&part.stream, cudaStreamNonBlocking) != cudaSuccess) {
            part.stream = nullptr;
            return set_err(ctx, NAV_BA_ERR_CUDA, "cudaStreamCreate failed");
        }
        std::swap(pbs[k].host, part.host);
        std::swap(pbs[k].dev, part.dev);
    }
    int launched = 0;
    struct SwapBack {
        PreparedBatch* pbs;
        nav_ba_ctx* ctx;
        ~SwapBack() {
            // nothing left in flight: every part's stream, also one whose upload was enqueued and
            // whose launch then failed (its copies still read that part's pinned staging)
            for (int k = 0; k < kSolveParts; ++k)
                if (ctx->parts[k].stream) cudaStreamSynchronize(ctx->parts[k].stream);
            for (int k = 0; k < kSolveParts; ++k) {
                std::swap(pbs[k].host, ctx->parts[k].host);
                std::swap(pbs[k].dev, ctx->parts[k].dev);
            }
        }
    } swap_back{pbs, ctx};
    // part boundaries at (k / parts)^2 of the batch: the first part (the largest windows, whose solves
    // are the longest) is small, so the device starts on it early; later parts grow while the device
    // is busy (4 parts: 1/16, 3/16, 5/16, 7/16)
    // NAVBA_PART_BOUNDS="<f1>,<f2>,<f3>" (fractions of the batch, increasing) sets the boundaries
    // instead (diagnostics)
    double fb[kSolveParts + 1];
    for (int k = 0; k <= kSolveParts; ++k) fb[k] = (double)(k * k) / (kSolveParts * kSolveParts);
    {
        const char* pb = getenv("NAVBA_PART_BOUNDS");
        double f1 = 0, f2 = 0, f3 = 0;
        if (pb && sscanf(pb, "%lf,%lf,%lf", &f1, &f2, &f3) == 3 && 0 < f1 && f1 < f2 && f2 < f3 && f3 < 1) {
            fb[1] = f1;
            fb[2] = f2;
            fb[3] = f3;
        }
    }
    auto part_lo = [&](int k) { return k >= kSolveParts ? n : (int)(n * fb[k]); };
    // the first part holds the largest windows and has the device nearly to itself until the later
    // parts are uploaded: each of its windows is solved by a cluster of CTAs, which shortens those
    // windows (the batch's critical path) and fills the otherwise idle SMs of the ramp.
    // NAVBA_PART0_SHAPE="<cluster>,<threads>" sets it (diagnostics).
    WindowLaunch part0_shape = kPart0Shape[o->precision == NAV_BA_FP64 ? 0 : 1];
    {
        const char* ps = getenv("NAVBA_PART0_SHAPE");
        int pc = 0, pt = 0;
        if (ps && sscanf(ps, "%d,%d", &pc, &pt) == 2 && (pc == 1 || pc == 2 || pc == 4 || pc == 8) &&
            (pt == 128 || pt == 256))
            part0_shape = WindowLaunch{pc, pt, 0.0};
    }
    double t_build = 0.0;
    // NAVBA_VERBOSE: the device timeline of the parts (upload start, kernel start and end per part)
    const char* verbose = getenv("NAVBA_VERBOSE");
    const bool timeline = verbose && verbose[0] == '1';
    struct Events {  // destroyed on every return
        cudaEvent_t ev[1 + 3 * kSolveParts] = {};
        ~Events() {
            for (auto& e : ev)
                if (e) cudaEventDestroy(e);
        }
    } tl;
    cudaEvent_t* tev = tl.ev;
    if (timeline) {
        for (auto& ev : tl.ev) cudaEventCreate(&ev);
        cudaEventRecord(tev[0], ctx->parts[0].stream);
    }
    for (int k = 0; k < kSolveParts; ++k) {
        const int lo = part_lo(k), hi = part_lo(k + 1);
        auto& part = ctx->parts[k];
        const auto tb = std::chrono::steady_clock::now();
        st = build_batch(ctx, pp.data() + lo, hi - lo, o, pbs[k]);
        t_build += ms_since(tb);
        if (st != NAV_BA_OK) {
            const nav_ba_status sc = check_batch(ctx, probs, n, o);
            return sc != NAV_BA_OK ? sc : st;
        }
        std::string why;
        if (timeline) cudaEventRecord(tev[1 + 3 * k], part.stream);
        // no wait for the copies: each part stages into its own pinned buffers, and every part's
        // stream is synchronized before the results are read (or on an error return)
        cudaError_t e = window_batch_upload(pbs[k], part.stream, o->precision, o->iterations + 1, part.stg, ctx->stg.pool,
                                            &why, false);
        if (e != cudaSuccess) return cuda_status(ctx, e, "upload");
        if (timeline) cudaEventRecord(tev[2 + 3 * k], part.stream);
        e = window_batch_launch(pbs[k], part.stream, o->precision, k == 0 ? part0_shape : ctx->shape[o->precision],
                                -1.0);
        if (e != cudaSuccess) return cuda_status(ctx, e, "window kernel");
        if (timeline) cudaEventRecord(tev[3 + 3 * k], part.stream);
        launched = k + 1;
    }
    const double t_setup = ms_since(t0);
    const auto t1 = std::chrono::steady_clock::now();
    // results in the parts' (size) order, then back to the caller's order
    std::vector<nav_ba_result> tp(n);
    for (int j = 0; j < n; ++j) {
        tp[j] = results[perm[j]];
        clear_stats(&tp[j]);
    }
    // each part is read back as soon as its own stream is done (the parts end in order: the first
    // holds the largest windows but started first), overlapping the later parts' kernels
    double t_solve = 0.0;
    for (int k = 0; k < kSolveParts; ++k) {
        const int lo = part_lo(k), hi = part_lo(k + 1);
        const auto tw = std::chrono::steady_clock::now();
        cudaError_t e = cudaStreamSynchronize(ctx->parts[k].stream);
        t_solve += ms_since(tw);
        if (e != cudaSuccess) return cuda_status(ctx, e, "window kernel");
        st = download_batch(ctx, pp.data() + lo, hi - lo, pbs[k], tp.data() + lo, &ctx->parts[k].stg, ctx->parts[k].stream);
        if (st != NAV_BA_OK && st != NAV_BA_EMPTY) return set_err(ctx, st, "a problem has a non-finite initial cost");
        for (int j = lo; j < hi; ++j) {
            if (pbs[k].host_status[j - lo] != kGridWindow) continue;
            st = solve_grid_window(ctx, pp[j], pbs[k].host[j - lo], *o, tp[j]);
            if (st != NAV_BA_OK) return st;
        }
    }
    const double t_down = ms_since(t1) - t_solve;
    if (timeline) {
        fprintf(stderr, "[navba host] %d problems in %d parts: build %.2f ms, setup (checks, build, stage, upload, "
                "launch; device already running) %.2f ms, wait %.2f ms, download %.2f ms\n", n, kSolveParts, t_build,
                t_setup, t_solve, t_down);
        for (int k = 0; k < launched; ++k) {
            float u = 0.f, ks = 0.f, ke = 0.f;
            cudaEventElapsedTime(&u, tev[0], tev[1 + 3 * k]);
            cudaEventElapsedTime(&ks, tev[0], tev[2 + 3 * k]);
            cudaEventElapsedTime(&ke, tev[0], tev[3 + 3 * k]);
            fprintf(stderr, "[navba host]   part %d (%d windows): upload from %.2f ms, kernel %.2f -> %.2f ms\n", k,
                    part_lo(k + 1) - part_lo(k), u, ks, ke);
        }
    }
    // byte counts of the whole call (each part's download reported its own)
    int64_t h2d = 0, d2h = 0;
    for (int k = 0; k < kSolveParts; ++k) {
        const int lo = part_lo(k), hi = part_lo(k + 1);
        h2d += pbs[k].dev.h2d_bytes;
        for (int j = lo; j < hi; ++j)
            if (pbs[k].host_status[j - lo] == NAV_BA_OK) {
                d2h += tp[j].d2h_bytes;
                break;
            }
    }
    for (int j = 0; j < n; ++j) {
        tp[j].time_setup_ms = t_setup;
        tp[j].time_solve_ms += t_solve;  // grid-engine problems already hold their own solve time
        tp[j].time_download_ms = t_down;
        tp[j].h2d_bytes = h2d;
        tp[j].d2h_bytes = d2h;
    }
    for (int j = 0; j < n; ++j) results[perm[j]] = tp[j];
    return NAV_BA_OK;
}

nav_ba_status solve_impl(nav_ba_ctx* ctx, const nav_ba_problem* probs, int n, const nav_ba_options* o,
                         nav_ba_result* results) {
    if (!ctx) return NAV_BA_ERR_ARGUMENT;
    if (!probs || !results || n < 0) return set_err(ctx, NAV_BA_ERR_ARGUMENT, "NULL argument");
    if (n >= kPipelineMinWindows && o && o->solver == NAV_BA_SOLVER_CHOLESKY)
        return solve_pipelined(ctx, probs, n, o, results);
    const auto t0 = std::chrono::steady_clock::now();
    PreparedBatch pb;
    // the context's host windows and device buffers are reused (their arrays keep their capacity)
    std::swap(pb.host, ctx->solve_host);
    std::swap(pb.dev, ctx->solve_dev);
    struct SwapBack {
        PreparedBatch& pb;
        nav_ba_ctx* ctx;
        ~SwapBack() {
            std::swap(pb.host, ctx->solve_host);
            std::swap(pb.dev, ctx->solve_dev);
        }
    } swap_back{pb, ctx};
    nav_ba_status st = build_batch(ctx, probs, n, o, pb);
    if (st != NAV_BA_OK) return st;
    const double t_build = ms_since(t0);
    std::string why;
    cudaError_t e = window_batch_upload(pb, ctx->stream, o->precision, o->iterations + 1, ctx->stg, ctx->stg.pool, &why);
    if (e != cudaSuccess) return cuda_status(ctx, e, "upload");
    const double t_setup = ms_since(t0);
    cudaEventRecord(ctx->ev0, ctx->stream);
    e = window_batch_launch(pb, ctx->stream, o->precision, ctx->shape[o->precision], -1.0);
    cudaEventRecord(ctx->ev1, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return cuda_status(ctx, e, "window kernel");
    float t_solve = 0.f;
    cudaEventElapsedTime(&t_solve, ctx->ev0, ctx->ev1);
    const auto t1 = std::chrono::steady_clock::now();
    std::vector<nav_ba_result> tmp(results, results + n);  // outputs untouched on error
    for (auto& r : tmp) clear_stats(&r);
    st = download_batch(ctx, probs, n, pb, tmp.data());
    if (st != NAV_BA_OK && st != NAV_BA_EMPTY) return set_err(ctx, st, "a problem has a non-finite initial cost");
    for (int i = 0; i < n; ++i) {
        if (pb.host_status[i] != kGridWindow) continue;
        st = solve_grid_window(ctx, probs[i], pb.host[i], *o, tmp[i]);
        if (st != NAV_BA_OK) return st;
    }
    const double t_down = ms_since(t1);
    const char* verbose = getenv("NAVBA_VERBOSE");
    if (verbose && verbose[0] == '1')
        fprintf(stderr, "[navba host] %d problems: build %.2f ms, stage+upload %.2f ms, device %.2f ms, download %.2f ms\n", n,
                t_build, t_setup - t_build, t_solve, t_down);
    for (int i = 0; i < n; ++i) {
        tmp[i].time_setup_ms = t_setup;
        tmp[i].time_solve_ms += t_solve;  // grid-engine problems already hold their own solve time
        tmp[i].time_download_ms = t_down;
        results[i] = tmp[i];
    }
    return NAV_BA_OK;
}

}  // namespace

extern "C" {

void nav_ba_options_default(nav_ba_options* o) {
    if (!o) return;
    std::memset(o, 0, sizeof(*o));
    o->iterations = 5;
    o->precision = NAV_BA_FP64;
    o->solver = NAV_BA_SOLVER_CHOLESKY;
    o->robust = 0;
    o->huber_delta = (double)(float)std::sqrt(5.99);
    o->initial_lambda = 0.0;
    o->tau = 1e-5;
    o->max_trials = 10;
    o->optimize_distortion = 0;
    o->pcg_tolerance = 1e-6;
    o->pcg_max_iterations = 100;
    o->deterministic = 1;
}

nav_ba_status nav_ba_create(nav_ba_ctx** out, int32_t device) {
    if (!out) return NAV_BA_ERR_ARGUMENT;
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) return NAV_BA_ERR_NO_DEVICE;
    if (device < 0 || device >= n) return NAV_BA_ERR_NO_DEVICE;
    if (cudaSetDevice(device) != cudaSuccess) return NAV_BA_ERR_NO_DEVICE;
    nav_ba_ctx* ctx = new nav_ba_ctx();
    ctx->device = device;
    if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreate(&ctx->ev0) != cudaSuccess || cudaEventCreate(&ctx->ev1) != cudaSuccess) {
        delete ctx;
        return NAV_BA_ERR_CUDA;
    }
    *out = ctx;
    return NAV_BA_OK;
}

void nav_ba_destroy(nav_ba_ctx* ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    window_batch_free(ctx->prepared.dev);
    window_batch_free(ctx->solve_dev);
    if (ctx->run_graph) cudaGraphExecDestroy(ctx->run_graph);
    for (auto& part : ctx->parts) {
        window_batch_free(part.dev);
        part.stg.release();
        if (part.stream) cudaStreamDestroy(part.stream);
    }
    ctx->pose.release();
    ctx->scratch.release();
    ctx->gws.release();
    ctx->stg.release();
    if (ctx->ev0) cudaEventDestroy(ctx->ev0);
    if (ctx->ev1) cudaEventDestroy(ctx->ev1);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
}

nav_ba_status nav_ba_solve(nav_ba_ctx* ctx, const nav_ba_problem* p, const nav_ba_options* o, nav_ba_result* r) {
    if (!ctx) return NAV_BA_ERR_ARGUMENT;
    if (!p || !o || !r) return set_err(ctx, NAV_BA_ERR_ARGUMENT, "NULL argument");
    cudaSetDevice(ctx->device);
    ctx->last_error.clear();
    std::string why;
    nav_ba_status st = validate_problem(p, &why);
    if (st != NAV_BA_OK) return set_err(ctx, st, why);
    nav_ba_result tmp = *r;
    st = solve_impl(ctx, p, 1, o, &tmp);
    if (st != NAV_BA_OK) return st;
    *r = tmp;
    return (nav_ba_status)(tmp.status == NAV_BA_EMPTY ? NAV_BA_EMPTY : NAV_BA_OK);
}

nav_ba_status nav_ba_solve_batched(nav_ba_ctx* ctx, const nav_ba_problem* windows, int32_t n,
                                   const nav_ba_options* o, nav_ba_result* results) {
    if (!ctx) return NAV_BA_ERR_ARGUMENT;
    cudaSetDevice(ctx->device);
    ctx->last_error.clear();
    return solve_impl(ctx, windows, n, o, results);
}

nav_ba_status nav_ba_prepare_batched(nav_ba_ctx* ctx, const nav_ba_problem* p, int32_t n, const nav_ba_options* o) {
    if (!ctx) return NAV_BA_ERR_ARGUMENT;
    if (!p || !o || n < 0) return set_err(ctx, NAV_BA_ERR_ARGUMENT, "NULL argument");
    cudaSetDevice(ctx->device);
    ctx->has_prepared = false;
    if (ctx->run_graph) {  // its buffers may be reallocated: captured again below
        cudaGraphExecDestroy(ctx->run_graph);
        ctx->run_graph = nullptr;
    }
    PreparedBatch& pb = ctx->prepared;
    pb.host.clear();
    pb.host_status.clear();
    pb.desc.clear();
    nav_ba_status st = build_batch(ctx, p, n, o, pb);
    if (st != NAV_BA_OK) return st;
    for (int i = 0; i < n; ++i)
        if (pb.host_status[i] == kGridWindow)
            return set_err(ctx, NAV_BA_ERR_UNSUPPORTED,
                           "nav_ba_prepare: problem " + std::to_string(i) + " exceeds the window engine (" +
                               std::to_string(kWinMaxFreeCams) + " free cameras); use nav_ba_solve");
    std::string why;
    cudaError_t e = window_batch_upload(pb, ctx->stream, o->precision, o->iterations + 1, ctx->stg, ctx->stg.pool, &why);
    if (e != cudaSuccess) return cuda_status(ctx, e, "upload");
    e = autotune(ctx, pb, o->precision);
    if (e != cudaSuccess) return cuda_status(ctx, e, "autotune");
    capture_run_graph(ctx, o->precision);
    ctx->prepared_problems.assign(p, p + n);
    ctx->prepared_opts = *o;
    ctx->has_prepared = true;
    return NAV_BA_OK;
}

nav_ba_status nav_ba_prepare(nav_ba_ctx* ctx, const nav_ba_problem* p, const nav_ba_options* o) {
    return nav_ba_prepare_batched(ctx, p, 1, o);
}

nav_ba_status nav_ba_fetch_batched(nav_ba_ctx* ctx, nav_ba_result* results) {
    if (!ctx) return NAV_BA_ERR_ARGUMENT;
    if (!ctx->has_prepared || !results) return set_err(ctx, NAV_BA_ERR_ARGUMENT, "nothing prepared");
    cudaSetDevice(ctx->device);
    const int n = (int)ctx->prepared_problems.size();
    std::vector<nav_ba_result> tmp(results, results + n);
    for (auto& r : tmp) clear_stats(&r);
    nav_ba_status st = download_batch(ctx, ctx->prepared_problems.data(), n, ctx->prepared, tmp.data());
    if (st != NAV_BA_OK && st != NAV_BA_EMPTY) return st;
    std::copy(tmp.begin(), tmp.end(), results);
    return NAV_BA_OK;
}

nav_ba_status nav_ba_run(nav_ba_ctx* ctx, const nav_ba_options* o, nav_ba_result* stats) {
    if (!ctx) return NAV_BA_ERR_ARGUMENT;
    if (!ctx->has_prepared) return set_err(ctx, NAV_BA_ERR_ARGUMENT, "nothing prepared");
    const nav_ba_options po = ctx->prepared_opts;
    if (o && (o->precision != po.precision || o->iterations != po.iterations))
        return set_err(ctx, NAV_BA_ERR_ARGUMENT, "run options must match the prepared precision and iterations");
    cudaSetDevice(ctx->device);
    if (o) ctx->prepared.lm = lm_options(*o);
    cudaEventRecord(ctx->ev0, ctx->stream);
    cudaError_t e;
    if (ctx->run_graph && std::memcmp(&ctx->graph_lm, &ctx->prepared.lm, sizeof(LmOptions)) == 0)
        e = cudaGraphLaunch(ctx->run_graph, ctx->stream);  // the launch captured at prepare time
    else
        e = window_batch_launch(ctx->prepared, ctx->stream, po.precision, ctx->shape[po.precision], -1.0);
    cudaEventRecord(ctx->ev1, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return cuda_status(ctx, e, "window kernel");
    window_phase_report(ctx->prepared, ctx->shape[po.precision], po.precision);
    if (stats) {
        float t = 0.f;
        cudaEventElapsedTime(&t, ctx->ev0, ctx->ev1);
        const int n = ctx->prepared.dev.n_win;
        std::vector<WinStats> ws(n);
        if (ctx->prepared.dev.n_queue > 0) {
            e = cudaMemcpy(ws.data(), ctx->prepared.dev.d_stats, sizeof(WinStats) * n, cudaMemcpyDeviceToHost);
            if (e != cudaSuccess) return cuda_status(ctx, e, "stats");
        }
        clear_stats(stats);
        stats->time_solve_ms = t;
        int64_t edge_iters = 0;
        for (int i = 0; i < n; ++i) {
            if (ctx->prepared.host_status[i] != NAV_BA_OK) continue;
            const WinStats& s = ws[i];
            stats->initial_cost += s.initial_cost;
            stats->final_cost += s.final_cost;
            stats->final_lambda = s.final_lambda;
            stats->iterations_done += s.iterations_done;
            stats->trials_accepted += s.accepted;
            stats->trials_rejected += s.rejected;
            stats->termination = s.termination;
            if (s.status != NAV_BA_OK) stats->status = s.status;
            stats->n_active_edges += ctx->prepared.host[i].ne;
            stats->n_free_cams += ctx->prepared.host[i].nfc;
            stats->n_free_points += ctx->prepared.host[i].nfp;
            stats->n_depth_nonpositive += s.depth_nonpos;
            edge_iters += (int64_t)ctx->prepared.host[i].ne * s.iterations_done;
        }
        stats->edge_iterations = edge_iters;
    }
    return NAV_BA_OK;
}

nav_ba_status nav_ba_fetch(nav_ba_ctx* ctx, nav_ba_result* r) {
    if (!ctx) return NAV_BA_ERR_ARGUMENT;
    if (!ctx->has_prepared || !r) return set_err(ctx, NAV_BA_ERR_ARGUMENT, "nothing prepared");
    cudaSetDevice(ctx->device);
    nav_ba_result tmp = *r;
    clear_stats(&tmp);
    nav_ba_status st = download_batch(ctx, ctx->prepared_problems.data(), 1, ctx->prepared, &tmp);
    if (st != NAV_BA_OK && st != NAV_BA_EMPTY) return st;
    *r = tmp;
    return NAV_BA_OK;
}

nav_ba_status nav_ba_linearize(nav_ba_ctx* ctx, const nav_ba_problem* p, const nav_ba_options* o, double* e,
                               double* jc, double* jp, double* w) {
    if (!ctx) return NAV_BA_ERR_ARGUMENT;
    if (!p || !o) return set_err(ctx, NAV_BA_ERR_ARGUMENT, "NULL argument");
    cudaSetDevice(ctx->device);
    std::string why;
    nav_ba_status st = validate_problem(p, &why);
    if (st != NAV_BA_OK) return set_err(ctx, st, why);
    st = validate_options(o, &why);
    if (st != NAV_BA_OK) return set_err(ctx, st, why);
    cudaError_t err = linearize_observations(*p, *o, ctx->stream, e, jc, jp, w, &why);
    return cuda_status(ctx, err, "linearize");
}

nav_ba_status nav_ba_reduced_system(nav_ba_ctx* ctx, const nav_ba_problem* p, const nav_ba_options* o, double lambda,
                                    int32_t capacity_free, int32_t* n_free, double* s, double* b, int32_t* cam_index) {
    if (!ctx) return NAV_BA_ERR_ARGUMENT;
    if (!p || !o || !n_free) return set_err(ctx, NAV_BA_ERR_ARGUMENT, "NULL argument");
    if (!(lambda >= 0)) return set_err(ctx, NAV_BA_ERR_ARGUMENT, "lambda must be >= 0");
    cudaSetDevice(ctx->device);
    PreparedBatch pb;
    nav_ba_options o1 = *o;
    o1.iterations = 1;
    nav_ba_status st = build_batch(ctx, p, 1, &o1, pb);
    if (st != NAV_BA_OK) return st;
    const HostWindow& h = pb.host[0];
    *n_free = h.nfc;
    if (cam_index) std::memcpy(cam_index, h.cam_free.data(), sizeof(int32_t) * p->n_cams);
    if (capacity_free < h.nfc || !s || !b) return NAV_BA_OK;
    if ((pb.host_status[0] != NAV_BA_OK && pb.host_status[0] != kGridWindow) || h.nfc == 0) {
        return NAV_BA_OK;
    }
    if (pb.host_status[0] == kGridWindow) {
        GridResult g;
        std::vector<double> dbg;
        cudaError_t e = grid_solve(h, lm_options(o1), intrinsics_of(*p), o1.precision, ctx->stream, &ctx->stg.pool,
                                   &ctx->gws, g, lambda, &dbg);
        if (e != cudaSuccess) return cuda_status(ctx, e, "reduced system");
        const int m = 6 * h.nfc;
        for (int r = 0; r < m; ++r)
            for (int c = 0; c < m; ++c) s[(size_t)r * m + c] = r >= c ? dbg[(size_t)r * m + c] : dbg[(size_t)c * m + r];
        std::memcpy(b, dbg.data() + (size_t)m * m, sizeof(double) * m);
        return NAV_BA_OK;
    }
    std::string why;
    std::swap(pb.dev, ctx->solve_dev);
    cudaError_t e = window_batch_upload(pb, ctx->stream, o1.precision, 2, ctx->stg, ctx->stg.pool, &why);
    if (e == cudaSuccess) e = window_batch_launch(pb, ctx->stream, o1.precision, ctx->shape[o1.precision], lambda);
    const int m = 6 * h.nfc;
    std::vector<double> out((size_t)m * m + m);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(out.data(), pb.dev.d_debug, sizeof(double) * out.size(), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    std::swap(pb.dev, ctx->solve_dev);
    if (e != cudaSuccess) return cuda_status(ctx, e, "reduced system");
    std::memcpy(s, out.data(), sizeof(double) * m * m);
    std::memcpy(b, out.data() + (size_t)m * m, sizeof(double) * m);
    return NAV_BA_OK;
}

nav_ba_status nav_ba_cost(nav_ba_ctx* ctx, const nav_ba_problem* p, const nav_ba_options* o, double* cost) {
    if (!ctx) return NAV_BA_ERR_ARGUMENT;
    if (!p || !o || !cost) return set_err(ctx, NAV_BA_ERR_ARGUMENT, "NULL argument");
    nav_ba_options o0 = *o;
    o0.iterations = 0;
    nav_ba_result r{};
    nav_ba_status st = nav_ba_solve(ctx, p, &o0, &r);
    if (st == NAV_BA_EMPTY) {
        *cost = 0.0;
        return NAV_BA_OK;
    }
    if (st != NAV_BA_OK) return st;
    *cost = r.initial_cost;
    return NAV_BA_OK;
}

nav_ba_status nav_ba_solve_noalloc(nav_ba_ctx* ctx, const nav_ba_problem* p, const nav_ba_options* o,
                                   nav_ba_result* r) {
    if (!ctx) return NAV_BA_ERR_ARGUMENT;
    if (!p || !o || !r) return set_err(ctx, NAV_BA_ERR_ARGUMENT, "NULL argument");
    cudaSetDevice(ctx->device);
    ctx->last_error.clear();
    std::string why;
    nav_ba_status st = validate_problem(p, &why);
    if (st == NAV_BA_OK) st = validate_options(o, &why);
    if (st != NAV_BA_OK) return set_err(ctx, st, why);
    nav_ba_result tmp = *r;
    clear_stats(&tmp);
    st = solve_window_noalloc(ctx->device, ctx->stream, *p, *o, tmp, &why);
    if (st == NAV_BA_EMPTY) {
        write_passthrough(*p, &tmp, false);
        tmp.termination = NAV_BA_TERM_NOTHING_TO_DO;
        tmp.status = NAV_BA_EMPTY;
        *r = tmp;
        return NAV_BA_EMPTY;
    }
    if (st != NAV_BA_OK) return set_err(ctx, st, why);
    *r = tmp;
    return NAV_BA_OK;
}

nav_ba_status nav_ba_solve_pose_batched(nav_ba_ctx* ctx, const nav_ba_pose_problem* probs, int32_t n,
                                        const nav_ba_options* o, nav_ba_pose_result* results) {
    if (!ctx) return NAV_BA_ERR_ARGUMENT;
    if ((!probs && n > 0) || !o || (!results && n > 0) || n < 0) return set_err(ctx, NAV_BA_ERR_ARGUMENT, "NULL argument");
    cudaSetDevice(ctx->device);
    std::string why;
    nav_ba_status st = validate_options(o, &why);
    if (st != NAV_BA_OK) return set_err(ctx, st, why);
    if (o->solver != NAV_BA_SOLVER_CHOLESKY || o->optimize_distortion)
        return set_err(ctx, NAV_BA_ERR_UNSUPPORTED, "motion-only BA solves its 6x6 system by Cholesky, without distortion");
    const auto t0 = std::chrono::steady_clock::now();
    std::vector<nav_ba_pose_result> tmp(results, results + n);  // outputs untouched on error
    float ms = 0.f;
    st = solve_pose_batch(ctx->stream, ctx->pose, probs, n, *o, tmp.data(), &ms, &why, ctx->stg);
    if (st != NAV_BA_OK) return set_err(ctx, st, why);
    for (int i = 0; i < n; ++i) results[i] = tmp[i];
    const char* verbose = getenv("NAVBA_VERBOSE");
    if (verbose && verbose[0] == '1')
        fprintf(stderr, "[navba pose] %d problems: kernel %.3f ms, call %.3f ms\n", n, ms,
                std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count());
    return NAV_BA_OK;
}

nav_ba_status nav_ba_twoview_check(nav_ba_ctx* ctx, const nav_ba_twoview* in, nav_ba_twoview_result* out) {
    if (!ctx) return NAV_BA_ERR_ARGUMENT;
    if (!in || !out) return set_err(ctx, NAV_BA_ERR_ARGUMENT, "NULL argument");
    cudaSetDevice(ctx->device);
    std::string why;
    const nav_ba_status st = twoview_check(ctx->stream, *in, *out, &why, ctx->scratch);
    if (st != NAV_BA_OK) return set_err(ctx, st, why);
    return NAV_BA_OK;
}

nav_ba_status nav_ba_undistort_points(nav_ba_ctx* ctx, const double* K, const double* dist, int32_t iterations,
                                      int32_t n, const double* uv_in, double* uv_out) {
    if (!ctx) return NAV_BA_ERR_ARGUMENT;
    cudaSetDevice(ctx->device);
    std::string why;
    const nav_ba_status st = undistort_points(ctx->stream, K, dist, iterations, n, uv_in, uv_out, &why, ctx->scratch);
    if (st != NAV_BA_OK) return set_err(ctx, st, why);
    return NAV_BA_OK;
}

nav_ba_status nav_ba_vjp(nav_ba_ctx* ctx, const nav_ba_problem* p, const nav_ba_options* o, nav_ba_schedule* sched,
                         const nav_ba_cotangent* cot, nav_ba_result* r, nav_ba_grads* grads) {
    if (!ctx) return NAV_BA_ERR_ARGUMENT;
    if (!p || !o || !sched || !r) return set_err(ctx, NAV_BA_ERR_ARGUMENT, "NULL argument");
    cudaSetDevice(ctx->device);
    std::string why;
    nav_ba_status st = validate_options(o, &why);
    if (st == NAV_BA_OK) st = validate_problem(p, &why);
    if (st != NAV_BA_OK) return set_err(ctx, st, why);
    if (o->precision != NAV_BA_FP64 || o->solver != NAV_BA_SOLVER_CHOLESKY || p->camera_model != NAV_BA_CAM_PINHOLE ||
        o->optimize_distortion)
        return set_err(ctx, NAV_BA_ERR_UNSUPPORTED,
                       "the VJP needs FP64 precision, the Cholesky solver and the pinhole model without distortion");
    GridVjp v;
    v.replay = sched->replay != 0;
    if (v.replay) {
        if (sched->n_steps < 0 || sched->n_steps > NAV_BA_VJP_MAX_STEPS)
            return set_err(ctx, NAV_BA_ERR_ARGUMENT, "schedule n_steps out of range");
        for (int s = 0; s < sched->n_steps; ++s)
            if (!std::isfinite(sched->lambda[s]) || sched->lambda[s] < 0.0)
                return set_err(ctx, NAV_BA_ERR_ARGUMENT, "schedule damping must be finite and >= 0");
        v.lambdas.assign(sched->lambda, sched->lambda + sched->n_steps);
    } else if (o->iterations > NAV_BA_VJP_MAX_STEPS) {
        return set_err(ctx, NAV_BA_ERR_UNSUPPORTED, "more LM iterations than NAV_BA_VJP_MAX_STEPS");
    }
    const bool bwd = cot && grads;
    v.backward = bwd;
    if (bwd) {
        if (!std::isfinite(cot->cost)) return set_err(ctx, NAV_BA_ERR_NONFINITE_INPUT, "non-finite cost cotangent");
        v.cost_bar = cot->cost;
        v.pose_bar = cot->cam_pose;
        v.point_bar = cot->points;
    }
    const auto t0 = std::chrono::steady_clock::now();
    HostWindow h;
    build_window(*p, *o, h);
    if (p->n_cams == 0 || h.ne == 0) {  // nothing is optimized: outputs are the inputs
        write_passthrough(*p, r, false);
        clear_stats(r);
        r->termination = NAV_BA_TERM_NOTHING_TO_DO;
        r->status = NAV_BA_EMPTY;
        if (!v.replay) sched->n_steps = 0;
        if (bwd) {
            if (grads->obs_uv) std::memset(grads->obs_uv, 0, sizeof(double) * 2 * p->n_obs);
            std::memset(grads->intrinsics, 0, sizeof(grads->intrinsics));
            if (grads->cam_tangent) std::memset(grads->cam_tangent, 0, sizeof(double) * 6 * p->n_cams);
            if (grads->points) std::memset(grads->points, 0, sizeof(double) * 3 * p->n_points);
        }
        return NAV_BA_EMPTY;
    }
    const double t_setup = ms_since(t0);
    GridResult g;
    cudaEventRecord(ctx->ev0, ctx->stream);
    cudaError_t e = grid_solve(h, lm_options(*o), intrinsics_of(*p), NAV_BA_FP64, ctx->stream, &ctx->stg.pool,
                               &ctx->gws, g, -1.0, nullptr, &v);
    cudaEventRecord(ctx->ev1, ctx->stream);
    if (e == cudaSuccess) e = cudaEventSynchronize(ctx->ev1);
    if (e != cudaSuccess) return cuda_status(ctx, e, "grid engine (vjp)");
    if (g.status != NAV_BA_OK)
        return set_err(ctx, (nav_ba_status)g.status, v.why.empty() ? std::string("non-finite initial cost") : v.why);
    float t = 0.f;
    cudaEventElapsedTime(&t, ctx->ev0, ctx->ev1);
    clear_stats(r);
    fill_grid_result(*p, h, *o, g, *r);
    r->time_setup_ms = t_setup;
    r->time_solve_ms = t;
    if (!v.replay) {
        sched->n_steps = (int32_t)v.lambdas.size();
        for (int s = 0; s < sched->n_steps; ++s) sched->lambda[s] = v.lambdas[s];
    }
    if (bwd) {
        if (grads->obs_uv) {
            std::memset(grads->obs_uv, 0, sizeof(double) * 2 * p->n_obs);
            for (int k = 0; k < h.ne; ++k) {
                grads->obs_uv[2LL * h.edge_obs[k]] = v.uv_bar[2LL * k];
                grads->obs_uv[2LL * h.edge_obs[k] + 1] = v.uv_bar[2LL * k + 1];
            }
        }
        std::memset(grads->intrinsics, 0, sizeof(grads->intrinsics));
        for (int k = 0; k < 4; ++k) grads->intrinsics[k] = v.intr_bar[k];
        if (grads->cam_tangent) std::memcpy(grads->cam_tangent, v.cam_bar.data(), sizeof(double) * 6 * p->n_cams);
        if (grads->points) std::memcpy(grads->points, v.pt_bar.data(), sizeof(double) * 3 * p->n_points);
    }
    return NAV_BA_OK;
}

const char* nav_ba_last_error(const nav_ba_ctx* ctx) { return ctx ? ctx->last_error.c_str() : ""; }

const char* nav_ba_status_string(nav_ba_status s) {
    switch (s) {
        case NAV_BA_OK: return "ok";
        case NAV_BA_EMPTY: return "empty problem: nothing to optimize";
        case NAV_BA_ERR_ARGUMENT: return "invalid argument";
        case NAV_BA_ERR_NONFINITE_INPUT: return "non-finite input";
        case NAV_BA_ERR_NONFINITE_COST: return "non-finite initial cost";
        case NAV_BA_ERR_CUDA: return "CUDA error";
        case NAV_BA_ERR_OUT_OF_MEMORY: return "out of memory";
        case NAV_BA_ERR_UNSUPPORTED: return "unsupported size or option";
        case NAV_BA_ERR_DEVICE_TIMEOUT: return "device wait timed out";
        case NAV_BA_ERR_NO_DEVICE: return "no CUDA device";
    }
    return "unknown status";
}

int32_t nav_ba_abi_version(void) { return NAV_BA_ABI_VERSION; }

}  // extern "C"
