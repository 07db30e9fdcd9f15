// Host graph build (nav24_gb300/csrc/structure.cpp, build_window) against a brute-force restatement
// on seeded random windows: active edges, the point-major edge order, free cameras and points, and
// the Schur pair and block counts (per-point camera masks up to 64 free cameras, pair loops beyond
// and for points a camera observes twice).  Prints "ok <windows>" or the first mismatch.
#include <cstdio>
#include <random>
#include <set>
#include <utility>
#include <vector>

#include "structure.hpp"

using namespace navba;

int main() {
    std::mt19937_64 rng(20261204);
    HostWindow w;
    int checked = 0;
    for (int t = 0; t < 2000; ++t) {
        const int nc = 1 + (int)(rng() % 90), np = 1 + (int)(rng() % 300);
        const int no = (int)(rng() % (6 * np + 1));
        std::vector<double> pose(12 * nc, 0.0), pts(3 * np, 1.0), uv(2 * no);
        for (int c = 0; c < nc; ++c) pose[12 * c] = pose[12 * c + 5] = pose[12 * c + 10] = 1.0;
        std::vector<int32_t> oc(no), op(no);
        std::vector<uint8_t> cf(nc), pf(np);
        const unsigned cfix = rng() % 4, pfix = rng() % 4;
        for (auto& x : cf) x = (rng() % 8) < cfix;
        for (auto& x : pf) x = (rng() % 8) < pfix;
        const int span = 1 + (int)(rng() % nc);
        for (int k = 0; k < no; ++k) {
            op[k] = (int)(rng() % np);
            oc[k] = (op[k] * 5 + (int)(rng() % span)) % nc;  // nearby cameras, repeats possible
            uv[2 * k] = (double)k;
            uv[2 * k + 1] = -(double)k;
        }
        nav_ba_problem p{};
        p.n_cams = nc;
        p.n_points = np;
        p.n_obs = no;
        p.cam_pose = pose.data();
        p.points = pts.data();
        p.obs_uv = uv.data();
        p.obs_cam = oc.data();
        p.obs_point = op.data();
        p.cam_fixed = cf.data();
        p.point_fixed = (t % 3) ? pf.data() : nullptr;
        p.camera_model = (t % 4 == 0) ? NAV_BA_CAM_PINHOLE_RADIAL : NAV_BA_CAM_PINHOLE;
        p.intrinsics[0] = p.intrinsics[1] = 500.0;
        nav_ba_options o{};
        o.optimize_distortion = (t % 8 == 0);
        build_window(p, o, w);
        // brute force
        const bool free_intr = o.optimize_distortion && p.camera_model == NAV_BA_CAM_PINHOLE_RADIAL;
        auto pfixed = [&](int i) { return p.point_fixed && p.point_fixed[i]; };
        std::vector<std::vector<int>> by_pt(np);  // active observations per point, in input order
        std::vector<char> cam_has(nc, 0);
        for (int k = 0; k < no; ++k)
            if (free_intr || !(cf[oc[k]] && pfixed(op[k]))) {
                by_pt[op[k]].push_back(k);
                cam_has[oc[k]] = 1;
            }
        std::vector<int> cfree(nc, -1);
        int nfc = 0;
        for (int c = 0; c < nc; ++c)
            if (!cf[c] && cam_has[c]) cfree[c] = nfc++;
        auto fail = [&](const char* what) {
            printf("mismatch %s (window %d: %d cameras, %d points, %d observations)\n", what, t, nc, np, no);
            return 1;
        };
        if (w.nfc != nfc) return fail("free cameras");
        for (int c = 0; c < nc; ++c)
            if (w.cam_free[c] != cfree[c]) return fail("free camera index");
        int e = 0, nfp = 0;
        int64_t pairs = 0;
        std::set<std::pair<int, int>> blocks;
        for (int i = 0; i < np; ++i) {
            if (w.pt_eoff[i] != e) return fail("point offsets");
            const int expect_free = (!pfixed(i) && !by_pt[i].empty()) ? nfp++ : -1;
            if (w.pt_free[i] != expect_free) return fail("free point index");
            for (int k : by_pt[i]) {
                if (w.edge_obs[e] != k || w.edge_cam[e] != oc[k] || w.edge_pt[e] != i || w.edge_uv[2 * e] != uv[2 * k])
                    return fail("edge order");
                ++e;
            }
            if (expect_free < 0) continue;
            for (int x : by_pt[i])
                for (int y : by_pt[i]) {
                    const int a = cfree[oc[x]], b = cfree[oc[y]];
                    if (a < 0 || b < 0 || b > a) continue;
                    ++pairs;
                    if (b < a) blocks.insert({a, b});
                }
        }
        if (w.ne != e || w.pt_eoff[np] != e) return fail("edge count");
        if (w.nfp != nfp) return fail("free points");
        if (w.n_pairs != pairs) return fail("Schur pairs");
        if (w.n_schur_blocks != nfc + (int)blocks.size()) return fail("Schur blocks");
        ++checked;
    }
    printf("ok %d\n", checked);
    return 0;
}
