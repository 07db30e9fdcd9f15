// noalloc.cu - nav_ba_solve_noalloc: one-window solve whose device memory is a fixed static array.
//
// Who needs it: callers that must not allocate device memory at solve time.  Examples are a
// tracking thread with a real-time budget (cudaMalloc and cudaFree can block for milliseconds and
// cudaFree synchronizes the device), a process whose device memory is already reserved by another
// framework's caching allocator (a raw cudaMalloc can fail or fragment that pool), and code that
// must keep its device footprint fixed and known up front.  This entry point solves one window with
// the same kernel as nav_ba_solve, but every device buffer it touches (staged inputs, scratch,
// staged outputs) is carved out of one file-scope __device__ array of NAV_BA_NOALLOC_ARENA_BYTES.
// Every GPU that loads the library holds that array until the process exits.  The call makes no
// cudaMalloc, cudaFree, cudaMallocAsync or cudaHostAlloc and uses no allocating library routine.
//
// The array is shared by every call on a device and keeps the previous call's contents: the
// kernel rewrites everything it reads before reading it, and this file clears the work-queue
// counter and the statistics on every call.  Two calls whose work overlaps on the GPU (for example
// from two contexts on the same device) race on the array.
#include <chrono>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "engine.hpp"

namespace navba {
namespace {

// The arena (device side).  Host code must not take its address directly: in host code the name
// stands for a host-side shadow, not device memory.  noalloc_arena() asks the runtime for the
// device address, once per device.
static __device__ __align__(256) unsigned char g_noalloc_arena[NAV_BA_NOALLOC_ARENA_BYTES];

constexpr int kMaxDevices = 64;
unsigned char* g_arena_ptr[kMaxDevices] = {};
std::mutex g_arena_mutex;

// Device address of the arena on the current device (set up on the first call per device).
cudaError_t noalloc_arena(int device, unsigned char** out) {
    if (device < 0 || device >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_arena_mutex);
    if (!g_arena_ptr[device]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_arena);
        if (e != cudaSuccess) return e;
        g_arena_ptr[device] = static_cast<unsigned char*>(p);
    }
    *out = g_arena_ptr[device];
    return cudaSuccess;
}

size_t up256(size_t x) { return (x + 255) & ~(size_t)255; }

}  // namespace

// Solve one window in the static arena.  Used by nav_ba_solve_noalloc (nav_ba_api.cu).
nav_ba_status solve_window_noalloc(int device, cudaStream_t stream, const nav_ba_problem& p,
                                   const nav_ba_options& o, nav_ba_result& r, std::string* why) {
    auto fail = [&](nav_ba_status st, const std::string& msg) {
        if (why) *why = msg;
        return st;
    };
    // host-clock timings (events would have to be created, which this call avoids)
    const auto t0 = std::chrono::steady_clock::now();
    auto ms_since = [](std::chrono::steady_clock::time_point t) {
        return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t).count();
    };
    if (o.solver != NAV_BA_SOLVER_CHOLESKY)
        return fail(NAV_BA_ERR_UNSUPPORTED, "the no-allocation solve uses the Cholesky solver");
    if (o.optimize_distortion && p.camera_model == NAV_BA_CAM_PINHOLE_RADIAL)
        return fail(NAV_BA_ERR_UNSUPPORTED, "the no-allocation solve does not optimize distortion");
    if (p.n_cams > NAV_BA_NOALLOC_MAX_CAMS || p.n_points > NAV_BA_NOALLOC_MAX_POINTS ||
        p.n_obs > NAV_BA_NOALLOC_MAX_OBS)
        return fail(NAV_BA_ERR_UNSUPPORTED,
                    "problem exceeds the no-allocation limits (" + std::to_string(NAV_BA_NOALLOC_MAX_CAMS) +
                        " cameras, " + std::to_string(NAV_BA_NOALLOC_MAX_POINTS) + " points, " +
                        std::to_string(NAV_BA_NOALLOC_MAX_OBS) + " observations)");
    PreparedBatch pb;
    pb.host.resize(1);
    pb.host_status.assign(1, NAV_BA_OK);
    build_window(p, o, pb.host[0]);
    const HostWindow& h = pb.host[0];
    if (p.n_cams == 0 || h.ne == 0) return NAV_BA_EMPTY;
    if (h.nfc > kWinMaxFreeCams)
        return fail(NAV_BA_ERR_UNSUPPORTED, "more than " + std::to_string(kWinMaxFreeCams) + " free cameras");
    if (h.n_pairs > NAV_BA_NOALLOC_MAX_PAIRS)
        return fail(NAV_BA_ERR_UNSUPPORTED, "more than " + std::to_string(NAV_BA_NOALLOC_MAX_PAIRS) +
                                                " Schur pairs (points seen by many cameras)");
    unsigned char* arena = nullptr;
    cudaError_t e = noalloc_arena(device, &arena);
    if (e != cudaSuccess) return fail(NAV_BA_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));

    // arena layout for this window
    const int64_t nc = h.ncam, np = h.npt, ne = h.ne, npair = h.n_pairs;
    const size_t rs = o.precision == NAV_BA_MIXED ? sizeof(float) : sizeof(double);
    const size_t rec = o.precision == NAV_BA_MIXED ? 20 : 18;
    const int trace_stride = o.iterations + 1;
    size_t off = 0;
    auto carve = [&](size_t bytes) {
        const size_t at = off;
        off += up256(std::max<size_t>(bytes, 16));
        return at;
    };
    const size_t o_win = carve(sizeof(WinDesc)), o_order = carve(sizeof(int32_t)), o_queue = carve(sizeof(int32_t));
    const size_t o_cam = carve(sizeof(CamState) * nc), o_cfree = carve(sizeof(int32_t) * nc);
    const size_t o_pinit = carve(sizeof(double) * 4 * np), o_pfree = carve(sizeof(int32_t) * np);
    const size_t o_peoff = carve(sizeof(int32_t) * (np + 1));
    const size_t o_ecam = carve(sizeof(int32_t) * ne), o_efc = carve(sizeof(int32_t) * ne);
    const size_t o_ept = carve(sizeof(int32_t) * ne), o_euv = carve(sizeof(double) * 2 * ne);
    const size_t o_x0 = carve(sizeof(double) * 4 * np), o_x1 = carve(sizeof(double) * 4 * np);
    const size_t o_vg = carve(rs * 12 * np), o_lt = carve(rs * 12 * np);
    const size_t o_w = carve(o.precision == NAV_BA_MIXED ? 16 : rs * rec * ne), o_a = carve(rs * rec * ne);
    const size_t eb = o.precision == NAV_BA_MIXED ? rs * 2 * ne : 16;
    const size_t o_e0 = carve(eb), o_e1 = carve(eb);
    const size_t o_list = carve(sizeof(int32_t) * ne);
    const size_t o_pairs = carve(sizeof(uint32_t) * npair);
    const size_t o_uvr = carve(o.precision == NAV_BA_MIXED ? rs * 2 * ne : 16);
    const size_t o_s = carve(o.precision == NAV_BA_MIXED ? sizeof(double) * (size_t)(6 * h.nfc) * (6 * h.nfc + 1) / 2 : 16);
    const size_t o_xr0 = carve(o.precision == NAV_BA_MIXED ? rs * 4 * np : 16);
    const size_t o_xr1 = carve(o.precision == NAV_BA_MIXED ? rs * 4 * np : 16);
    const size_t o_cout = carve(sizeof(CamState) * nc), o_pout = carve(sizeof(double) * 4 * np);
    const size_t o_trace = carve(sizeof(double) * trace_stride), o_stats = carve(sizeof(WinStats));
    if (off > (size_t)NAV_BA_NOALLOC_ARENA_BYTES)
        return fail(NAV_BA_ERR_UNSUPPORTED, "problem needs " + std::to_string(off) + " bytes of the " +
                                                std::to_string((size_t)NAV_BA_NOALLOC_ARENA_BYTES) +
                                                "-byte no-allocation arena");
    WindowBatch& b = pb.dev;
    b.d_win = reinterpret_cast<WinDesc*>(arena + o_win);
    b.d_order = reinterpret_cast<int32_t*>(arena + o_order);
    b.d_queue = reinterpret_cast<int32_t*>(arena + o_queue);
    b.d_cam_init = reinterpret_cast<CamState*>(arena + o_cam);
    b.d_cam_free = reinterpret_cast<int32_t*>(arena + o_cfree);
    b.d_pt_init = reinterpret_cast<double*>(arena + o_pinit);
    b.d_pt_free = reinterpret_cast<int32_t*>(arena + o_pfree);
    b.d_pt_eoff = reinterpret_cast<int32_t*>(arena + o_peoff);
    b.d_edge_cam = reinterpret_cast<int32_t*>(arena + o_ecam);
    b.d_edge_fc = reinterpret_cast<int32_t*>(arena + o_efc);
    b.d_edge_pt = reinterpret_cast<int32_t*>(arena + o_ept);
    b.d_edge_uv = reinterpret_cast<double*>(arena + o_euv);
    b.d_x[0] = reinterpret_cast<double*>(arena + o_x0);
    b.d_x[1] = reinterpret_cast<double*>(arena + o_x1);
    b.d_pt_vg = arena + o_vg;
    b.d_pt_lt = arena + o_lt;
    b.d_edge_w = arena + o_w;
    b.d_edge_a = arena + o_a;
    b.d_edge_e[0] = arena + o_e0;
    b.d_edge_e[1] = arena + o_e1;
    b.d_cam_list = reinterpret_cast<int32_t*>(arena + o_list);
    b.d_edge_uvr = arena + o_uvr;
    b.d_s = reinterpret_cast<double*>(arena + o_s);
    b.d_xr[0] = arena + o_xr0;
    b.d_xr[1] = arena + o_xr1;
    b.d_pairs = reinterpret_cast<uint32_t*>(arena + o_pairs);
    b.d_cam_out = reinterpret_cast<CamState*>(arena + o_cout);
    b.d_pt_out = reinterpret_cast<double*>(arena + o_pout);
    b.d_trace = reinterpret_cast<double*>(arena + o_trace);
    b.d_stats = reinterpret_cast<WinStats*>(arena + o_stats);
    b.d_debug = nullptr;
    b.d_phase = nullptr;
    b.n_win = 1;
    b.n_queue = 1;
    b.ncam = nc; b.npt = np; b.ne = ne; b.npair = npair;
    b.max_m = 6 * h.nfc;
    b.max_ncam = h.ncam;
    b.precision = o.precision;
    b.trace_stride = trace_stride;

    // host-side staging (pageable host memory; the runtime copies it)
    WinDesc d{};
    d.cam0 = 0; d.ncam = h.ncam; d.pt0 = 0; d.npt = h.npt; d.e0 = 0; d.ne = h.ne;
    d.nfc = h.nfc; d.nfp = h.nfp; d.pair0 = 0; d.npair = h.n_pairs; d.s0 = 0;
    pb.desc.assign(1, d);
    const int32_t order0 = 0;
    std::vector<int32_t> edge_fc(ne);
    for (int64_t k = 0; k < ne; ++k) edge_fc[k] = h.cam_free[h.edge_cam[k]];
    pb.lm.iterations = o.iterations;
    pb.lm.max_trials = o.max_trials;
    pb.lm.robust = o.robust;
    pb.lm.huber_delta = o.huber_delta;
    pb.lm.initial_lambda = o.initial_lambda;
    pb.lm.tau = o.tau;
    pb.intr = make_intr(p.intrinsics, p.camera_model);
    int64_t h2d = 0, d2h = 0;
    auto up = [&](void* dst, const void* src, size_t bytes) {
        if (e != cudaSuccess || bytes == 0) return;
        e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, stream);
        h2d += (int64_t)bytes;
    };
    up(b.d_win, &d, sizeof(WinDesc));
    up(b.d_order, &order0, sizeof(int32_t));
    up(b.d_cam_init, h.cam.data(), sizeof(CamState) * nc);
    up(b.d_cam_free, h.cam_free.data(), sizeof(int32_t) * nc);
    up(b.d_pt_init, h.pt.data(), sizeof(double) * 4 * np);
    up(b.d_pt_free, h.pt_free.data(), sizeof(int32_t) * np);
    up(b.d_pt_eoff, h.pt_eoff.data(), sizeof(int32_t) * (np + 1));
    up(b.d_edge_cam, h.edge_cam.data(), sizeof(int32_t) * ne);
    up(b.d_edge_fc, edge_fc.data(), sizeof(int32_t) * ne);
    up(b.d_edge_pt, h.edge_pt.data(), sizeof(int32_t) * ne);
    up(b.d_edge_uv, h.edge_uv.data(), sizeof(double) * 2 * ne);
    // the arena keeps the previous call's contents: clear the statistics (the queue counter is
    // reset by the launch itself)
    if (e == cudaSuccess) e = cudaMemsetAsync(b.d_stats, 0, sizeof(WinStats), stream);
    // setup: host structure and the enqueued uploads; solve: until the kernel has finished
    const double t_setup = ms_since(t0);
    const auto t1 = std::chrono::steady_clock::now();
    if (e == cudaSuccess) e = window_batch_launch(pb, stream, o.precision, WindowLaunch{1, 256}, -1.0);
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    const double t_solve = ms_since(t1);
    const auto t2 = std::chrono::steady_clock::now();
    std::vector<CamState> cams(nc);
    std::vector<double> pts(4 * np), trace(trace_stride);
    WinStats st{};
    auto dn = [&](void* dst, const void* src, size_t bytes) {
        if (e != cudaSuccess || bytes == 0) return;
        e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, stream);
        d2h += (int64_t)bytes;
    };
    dn(cams.data(), b.d_cam_out, sizeof(CamState) * nc);
    dn(pts.data(), b.d_pt_out, sizeof(double) * 4 * np);
    dn(trace.data(), b.d_trace, sizeof(double) * trace_stride);
    dn(&st, b.d_stats, sizeof(WinStats));
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    if (e != cudaSuccess) return fail(NAV_BA_ERR_CUDA, std::string("no-allocation solve: ") + cudaGetErrorString(e));
    if (st.status != NAV_BA_OK)
        return fail((nav_ba_status)st.status,
                    std::string("no-allocation solve: ") + nav_ba_status_string((nav_ba_status)st.status));
    r.initial_cost = st.initial_cost;
    r.final_cost = st.final_cost;
    r.final_lambda = st.final_lambda;
    r.iterations_done = st.iterations_done;
    r.trials_accepted = st.accepted;
    r.trials_rejected = st.rejected;
    r.termination = st.termination;
    r.n_active_edges = h.ne;
    r.n_free_cams = h.nfc;
    r.n_free_points = h.nfp;
    r.n_schur_blocks = h.n_schur_blocks;
    r.edge_iterations = (int64_t)h.ne * st.iterations_done;
    r.n_depth_nonpositive = st.depth_nonpos;
    r.h2d_bytes = h2d;
    r.d2h_bytes = d2h;
    r.time_setup_ms = t_setup;
    r.time_solve_ms = t_solve;
    r.status = NAV_BA_OK;
    if (r.cam_pose_out)
        for (int c = 0; c < p.n_cams; ++c) pose12_from_cam(cams[c], r.cam_pose_out + 12LL * c);
    if (r.points_out)
        for (int k = 0; k < p.n_points; ++k)
            for (int j = 0; j < 3; ++j) r.points_out[3LL * k + j] = pts[4LL * k + j];
    if (r.intrinsics_out) std::memcpy(r.intrinsics_out, p.intrinsics, sizeof(double) * 8);
    if (r.cost_trace)
        for (int k = 0; k <= st.iterations_done; ++k) r.cost_trace[k] = trace[k];
    r.time_download_ms = ms_since(t2);
    return NAV_BA_OK;
}

}  // namespace navba
