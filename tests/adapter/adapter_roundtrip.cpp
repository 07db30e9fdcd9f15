// Test program: builds nav24 objects (frames, KeyPoint2D observations, Point3D map points, a
// pinhole Calibration) from a binary problem file, solves with BE::GraphOptimGpu exactly as
// nav24's call sites do (PR_VBA + solve), and writes what the solve mutated: every frame's pose
// (3x4) and optId, every point's position.
//
// input : int32[8] {n_cams, n_points, n_obs, iterations, robust, precision, edge_cases, 0}
//         float64[4] fx fy cx cy; float64[n_cams*12] poses; float64[n_points*3] points;
//         float64[n_obs*2] undistorted measurements; int32[n_cams] fixed; int32[n_points] fixed;
//         int32[n_obs] camera; int32[n_obs] point
// output: int32[2] {status, termination}; float64[n_cams*12] poses (NaN for a frame without pose);
//         uint64[n_cams] optIds; float64[n_points*3] points; float64[2] {initial cost, final cost}
//
// edge_cases = 1 builds the graph-assembly cases that GraphOptim filters (BE_GraphOptim.cpp:87-89,
// 143-144, 160-172, 204-205), by fixed index patterns that tests/test_adapter.py restates:
//   camera kNoPoseCam has no pose (and optId -1, as a previous solve leaves it);
//   observation k: k % 13 == 0 invalid; k % 11 == 1 a plain Point2D (not a KeyPoint2D);
//   k % 17 == 5 belongs to frame A outside the problem, optId 0 (its edge goes to pose vertex 0, as
//   g2o's vertex(0) lookup does); else k % 19 == 7 to frame B outside the problem, optId -1;
//   point i: i % 50 == 7 invalid; i % 97 == 3 every observation invalid (the point has no edge);
//   frame 1's observation list also holds a null pointer.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <memory>
#include <vector>

#include "Calibration.hpp"
#include "Frame.hpp"
#include "GraphOptimGpu.hpp"
#include "Point2D.hpp"
#include "Point3D.hpp"

using namespace NAV24;

template <class T>
static std::vector<T> rd(FILE* f, size_t n) {
    std::vector<T> v(n);
    if (n && fread(v.data(), sizeof(T), n, f) != n) {
        fprintf(stderr, "short read\n");
        exit(2);
    }
    return v;
}

int main(int argc, char** argv) {
    if (argc != 3) {
        fprintf(stderr, "usage: %s in.bin out.bin\n", argv[0]);
        return 2;
    }
    FILE* fi = fopen(argv[1], "rb");
    if (!fi) return 2;
    const auto hdr = rd<int32_t>(fi, 8);
    const int nc = hdr[0], np = hdr[1], no = hdr[2];
    const auto K = rd<double>(fi, 4);
    const auto pose = rd<double>(fi, 12LL * nc);
    const auto pts = rd<double>(fi, 3LL * np);
    const auto uv = rd<double>(fi, 2LL * no);
    const auto cfix = rd<int32_t>(fi, nc);
    const auto pfix = rd<int32_t>(fi, np);
    const auto oc = rd<int32_t>(fi, no);
    const auto op = rd<int32_t>(fi, no);
    fclose(fi);

    const bool edge_cases = hdr[6] != 0;
    constexpr int kNoPoseCam = 3;
    const unsigned long kNoVertex = (unsigned long)-1;
    std::vector<FramePtr> frames;
    std::vector<std::vector<OB::ObsPtr>> frame_obs(nc);
    for (int c = 0; c < nc; ++c) {
        Eigen::Matrix4d T = Eigen::Matrix4d::Identity();
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 4; ++j) T(i, j) = pose[12LL * c + 4 * i + j];
        PosePtr P = std::make_shared<TF::PoseSE3>("w", "c" + std::to_string(c), 0.1 * c, T);
        if (edge_cases && c == kNoPoseCam) P = nullptr;
        auto f = std::make_shared<Frame>(0.1 * c, P, std::vector<OB::ObsPtr>{});
        f->setOptFixed(cfix[c] != 0);
        if (edge_cases && c == kNoPoseCam) f->setOptId(kNoVertex);
        frames.push_back(f);
    }
    // frames outside the problem: A with optId 0 (never optimized), B with optId -1
    auto frameA = std::make_shared<Frame>(-1.0, nullptr, std::vector<OB::ObsPtr>{});
    auto frameB = std::make_shared<Frame>(-2.0, nullptr, std::vector<OB::ObsPtr>{});
    frameB->setOptId(kNoVertex);
    std::vector<OB::ObsPtr> obsA, obsB;
    std::vector<std::shared_ptr<WO::Point3D>> points;
    for (int i = 0; i < np; ++i) {
        auto p = std::make_shared<WO::Point3D>(pts[3LL * i], pts[3LL * i + 1], pts[3LL * i + 2]);
        p->setOptFixed(pfix[i] != 0);
        if (edge_cases && i % 50 == 7) p->setValid(false);
        points.push_back(p);
    }
    for (int k = 0; k < no; ++k) {
        const cv::Point2f z((float)uv[2LL * k], (float)uv[2LL * k + 1]);
        std::shared_ptr<OB::Point2D> o;
        if (edge_cases && k % 11 == 1) {
            o = std::make_shared<OB::Point2D>(z.x, z.y);
        } else {
            cv::KeyPoint kp;
            kp.pt = z;
            o = std::make_shared<OB::KeyPoint2D>(kp, cv::Mat());
        }
        o->setPointUd(z);
        if (edge_cases && (k % 13 == 0 || op[k] % 97 == 3)) o->setValid(false);
        o->setWorldObject(points[op[k]]);
        points[op[k]]->addObservation(o);
        if (edge_cases && k % 17 == 5) {
            o->setFrame(frameA);
            obsA.push_back(o);
        } else if (edge_cases && k % 19 == 7) {
            o->setFrame(frameB);
            obsB.push_back(o);
        } else {
            o->setFrame(frames[oc[k]]);
            frame_obs[oc[k]].push_back(o);
        }
    }
    if (edge_cases) frame_obs[1].insert(frame_obs[1].begin() + frame_obs[1].size() / 2, OB::ObsPtr());
    for (int c = 0; c < nc; ++c) frames[c]->setObservations(frame_obs[c]);
    frameA->setObservations(obsA);
    frameB->setObservations(obsB);

    auto calib = std::make_shared<Calibration>((float)K[0], (float)K[1], (float)K[2], (float)K[3]);
    auto problem = std::make_shared<PR_VBA>(frames, calib);
    problem->setNumIter(hdr[3]);
    problem->mbRobust = hdr[4] != 0;
    auto solver = std::make_shared<BE::GraphOptimGpu>(0, hdr[5]);
    solver->solve(problem);

    FILE* fo = fopen(argv[2], "wb");
    const nav_ba_result* r = solver->lastResults().empty() ? nullptr : &solver->lastResults()[0];
    const int32_t st[2] = {(int32_t)solver->lastStatus(), r ? r->termination : -1};
    fwrite(st, sizeof(int32_t), 2, fo);
    for (int c = 0; c < nc; ++c) {
        Eigen::Matrix4d T = Eigen::Matrix4d::Identity();
        const bool has_pose = frames[c]->getPose() != nullptr;
        if (has_pose) T = frames[c]->getPose()->getPose();
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 4; ++j) {
                const double v = has_pose ? T(i, j) : std::nan("");
                fwrite(&v, sizeof(double), 1, fo);
            }
    }
    for (int c = 0; c < nc; ++c) {
        const uint64_t id = frames[c]->getOptId();
        fwrite(&id, sizeof(uint64_t), 1, fo);
    }
    for (int i = 0; i < np; ++i) {
        const auto& p = points[i]->getPoint();
        const double v[3] = {p.x, p.y, p.z};
        fwrite(v, sizeof(double), 3, fo);
    }
    const double costs[2] = {r ? r->initial_cost : 0.0, r ? r->final_cost : 0.0};
    fwrite(costs, sizeof(double), 2, fo);
    fclose(fo);
    if (solver->lastStatus() != NAV_BA_OK) fprintf(stderr, "solve status %d: %s\n", solver->lastStatus(), solver->lastError());
    return solver->lastStatus() == NAV_BA_OK ? 0 : 1;
}
