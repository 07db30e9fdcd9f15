// structure.cpp - host-side graph build (see structure.hpp).
#include "structure.hpp"

#include <algorithm>
#include <cmath>

namespace navba {

// x * 0 is 0 for every finite x and NaN for NaN and +-Inf, so sums of x * 0 in independent
// accumulators are 0 exactly when every value is finite (branch-free: the loop vectorizes).
static bool all_finite(const double* a, long long n) {
    double acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    long long i = 0;
    for (; i + 8 <= n; i += 8)
        for (int k = 0; k < 8; ++k) acc[k] += a[i + k] * 0.0;
    for (; i < n; ++i) acc[0] += a[i] * 0.0;
    double t = 0.0;
    for (int k = 0; k < 8; ++k) t += acc[k];
    return t == 0.0;
}

// Every index in [0, bound) (branch-free).
static bool all_below(const int32_t* v, long long n, int32_t bound) {
    uint32_t bad = 0;
    for (long long i = 0; i < n; ++i) bad |= (uint32_t)v[i] >= (uint32_t)bound;
    return bad == 0;
}

nav_ba_status validate_problem(const nav_ba_problem* p, std::string* why) {
    auto fail = [&](nav_ba_status s, const char* msg) {
        if (why) *why = msg;
        return s;
    };
    if (!p) return fail(NAV_BA_ERR_ARGUMENT, "problem is NULL");
    if (p->n_cams < 0 || p->n_points < 0 || p->n_obs < 0) return fail(NAV_BA_ERR_ARGUMENT, "negative size");
    if ((p->n_cams && !p->cam_pose) || (p->n_points && !p->points) ||
        (p->n_obs && (!p->obs_uv || !p->obs_cam || !p->obs_point)))
        return fail(NAV_BA_ERR_ARGUMENT, "NULL array with nonzero size");
    if (p->camera_model != NAV_BA_CAM_PINHOLE && p->camera_model != NAV_BA_CAM_PINHOLE_RADIAL &&
        p->camera_model != NAV_BA_CAM_KANNALA_BRANDT8)
        return fail(NAV_BA_ERR_ARGUMENT, "unknown camera model");
    if (!all_below(p->obs_cam, p->n_obs, p->n_cams) || !all_below(p->obs_point, p->n_obs, p->n_points))
        return fail(NAV_BA_ERR_ARGUMENT, "observation index out of range");
    if (!all_finite(p->cam_pose, 12LL * p->n_cams) || !all_finite(p->points, 3LL * p->n_points) ||
        !all_finite(p->obs_uv, 2LL * p->n_obs) || !all_finite(p->intrinsics, 8))
        return fail(NAV_BA_ERR_NONFINITE_INPUT, "non-finite input value");
    return NAV_BA_OK;
}

nav_ba_status validate_options(const nav_ba_options* o, std::string* why) {
    auto fail = [&](const char* msg) {
        if (why) *why = msg;
        return NAV_BA_ERR_ARGUMENT;
    };
    if (!o) return fail("options is NULL");
    if (o->iterations < 0) return fail("iterations < 0");
    if (o->max_trials < 1) return fail("max_trials < 1");
    if (o->robust && !(o->huber_delta > 0)) return fail("huber_delta must be > 0");
    if (o->precision != NAV_BA_FP64 && o->precision != NAV_BA_MIXED) return fail("unknown precision");
    if (o->solver != NAV_BA_SOLVER_CHOLESKY && o->solver != NAV_BA_SOLVER_PCG) return fail("unknown solver");
    if (!(o->tau >= 0) || !std::isfinite(o->initial_lambda)) return fail("invalid damping parameters");
    return NAV_BA_OK;
}

void build_window(const nav_ba_problem& p, const nav_ba_options& o, HostWindow& w) {
    const bool free_intr = o.optimize_distortion && p.camera_model == NAV_BA_CAM_PINHOLE_RADIAL;
    w.ncam = p.n_cams;
    w.npt = p.n_points;
    auto cam_fixed = [&](int c) { return p.cam_fixed && p.cam_fixed[c]; };
    auto pt_fixed = [&](int i) { return p.point_fixed && p.point_fixed[i]; };
    // active edges, counted per point (counting sort keeps input order within a point), and the
    // cameras with an active edge: the free cameras are known before the edges are placed
    auto active = [&](int c, int i) { return free_intr || !(cam_fixed(c) && pt_fixed(i)); };
    std::vector<int32_t> cnt(w.npt + 1, 0);
    std::vector<uint8_t> cam_has(w.ncam, 0);
    for (int k = 0; k < p.n_obs; ++k) {
        const int c = p.obs_cam[k], i = p.obs_point[k];
        if (active(c, i)) {
            cnt[i + 1]++;
            cam_has[c] = 1;
        }
    }
    w.pt_eoff.assign(w.npt + 1, 0);
    for (int i = 0; i < w.npt; ++i) w.pt_eoff[i + 1] = w.pt_eoff[i] + cnt[i + 1];
    w.ne = w.pt_eoff[w.npt];
    w.cam_free.assign(w.ncam, -1);
    w.nfc = 0;
    for (int c = 0; c < w.ncam; ++c)
        if (!cam_fixed(c) && cam_has[c]) w.cam_free[c] = w.nfc++;
    // edges point-major; up to 64 free cameras each point's mask of free cameras and whether one
    // of them observes it twice come along (for the Schur counts below)
    w.edge_cam.resize(w.ne);
    w.edge_obs.resize(w.ne);
    w.edge_uv.resize(2LL * w.ne);
    w.edge_pt.resize(w.ne);
    const bool masks = w.nfc > 0 && w.nfc <= 64;
    std::vector<uint64_t> pmask(masks ? w.npt : 0, 0);
    std::vector<uint8_t> prep(masks ? w.npt : 0, 0);
    std::vector<int32_t> fill(w.pt_eoff.begin(), w.pt_eoff.end() - 1);
    for (int k = 0; k < p.n_obs; ++k) {
        const int c = p.obs_cam[k], i = p.obs_point[k];
        if (!active(c, i)) continue;
        const int e = fill[i]++;
        w.edge_cam[e] = c;
        w.edge_obs[e] = k;
        w.edge_pt[e] = i;
        w.edge_uv[2LL * e] = p.obs_uv[2LL * k];
        w.edge_uv[2LL * e + 1] = p.obs_uv[2LL * k + 1];
        if (masks) {
            const int a = w.cam_free[c];
            if (a >= 0) {
                const uint64_t bit = 1ull << a;
                prep[i] |= (uint8_t)((pmask[i] & bit) != 0);
                pmask[i] |= bit;
            }
        }
    }
    w.pt_free.assign(w.npt, -1);
    w.nfp = 0;
    for (int i = 0; i < w.npt; ++i)
        if (!pt_fixed(i) && w.pt_eoff[i + 1] > w.pt_eoff[i]) w.pt_free[i] = w.nfp++;
    w.cam.resize(w.ncam);
    for (int c = 0; c < w.ncam; ++c) cam_from_pose12(p.cam_pose + 12LL * c, w.cam[c]);
    w.pt.assign(4LL * w.npt, 0.0);
    for (int i = 0; i < w.npt; ++i)
        for (int k = 0; k < 3; ++k) w.pt[4LL * i + k] = p.points[3LL * i + k];
    // Schur pairs (same free point, free cameras, b <= a) and the distinct lower blocks they touch.
    // Up to 64 free cameras: per point the mask of its free cameras gives k(k+1)/2 pairs (when no
    // camera observes the point twice) and each row's lower blocks by an OR; beyond, or with a
    // repeated camera, the pairs are counted one by one.
    w.n_pairs = 0;
    w.n_schur_blocks = w.nfc;  // the diagonal blocks
    if (masks) {
        std::vector<uint64_t> row(w.nfc, 0);  // row a: cameras b < a sharing a point with a
        for (int i = 0; i < w.npt; ++i) {
            if (w.pt_free[i] < 0) continue;
            const uint64_t m = pmask[i];
            if (!prep[i]) {
                const int64_t k = __builtin_popcountll(m);
                w.n_pairs += k * (k + 1) / 2;
            } else {
                for (int e = w.pt_eoff[i]; e < w.pt_eoff[i + 1]; ++e) {
                    const int a = w.cam_free[w.edge_cam[e]];
                    if (a < 0) continue;
                    for (int f = w.pt_eoff[i]; f < w.pt_eoff[i + 1]; ++f) {
                        const int b = w.cam_free[w.edge_cam[f]];
                        if (b >= 0 && b <= a) ++w.n_pairs;
                    }
                }
            }
            for (uint64_t r = m; r; r &= r - 1) {
                const int a = __builtin_ctzll(r);
                row[a] |= m & ((1ull << a) - 1);
            }
        }
        for (int a = 0; a < w.nfc; ++a) w.n_schur_blocks += __builtin_popcountll(row[a]);
    } else if (w.nfc > 0) {
        std::vector<uint8_t> seen((size_t)w.nfc * w.nfc, 0);
        std::vector<int32_t> fc;
        for (int i = 0; i < w.npt; ++i) {
            if (w.pt_free[i] < 0) continue;
            fc.clear();
            for (int e = w.pt_eoff[i]; e < w.pt_eoff[i + 1]; ++e) {
                const int a = w.cam_free[w.edge_cam[e]];
                if (a >= 0) fc.push_back(a);
            }
            for (size_t x = 0; x < fc.size(); ++x)
                for (size_t y = 0; y < fc.size(); ++y) {
                    const int a = fc[x], b = fc[y];
                    if (b > a) continue;
                    ++w.n_pairs;
                    if (b < a && !seen[(size_t)a * w.nfc + b]) {
                        seen[(size_t)a * w.nfc + b] = 1;
                        ++w.n_schur_blocks;
                    }
                }
        }
    }
}

}  // namespace navba
