// Test program: builds nav24 objects (frames, KeyPoint2D observations, Point3D map points, a
// pinhole Calibration) from a binary problem file, solves with BE::GraphOptimGpu exactly as
// nav24's call sites do (PR_VBA + solve), and writes what the solve mutated: every frame's pose
// (3x4) and optId, every point's position.
//
// input : int32[8] {n_cams, n_points, n_obs, iterations, robust, precision, 0, 0}
//         float64[4] fx fy cx cy; float64[n_cams*12] poses; float64[n_points*3] points;
//         float64[n_obs*2] undistorted measurements; int32[n_cams] fixed; int32[n_points] fixed;
//         int32[n_obs] camera; int32[n_obs] point
// output: int32[2] {status, termination}; float64[n_cams*12] poses; uint64[n_cams] optIds;
//         float64[n_points*3] points; float64[2] {initial cost, final cost}
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

    std::vector<FramePtr> frames;
    std::vector<std::vector<OB::ObsPtr>> frame_obs(nc);
    for (int c = 0; c < nc; ++c) {
        Eigen::Matrix4d T = Eigen::Matrix4d::Identity();
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 4; ++j) T(i, j) = pose[12LL * c + 4 * i + j];
        auto f = std::make_shared<Frame>(0.1 * c, std::make_shared<TF::PoseSE3>("w", "c" + std::to_string(c), 0.1 * c, T),
                                         std::vector<OB::ObsPtr>{});
        f->setOptFixed(cfix[c] != 0);
        frames.push_back(f);
    }
    std::vector<std::shared_ptr<WO::Point3D>> points;
    for (int i = 0; i < np; ++i) {
        auto p = std::make_shared<WO::Point3D>(pts[3LL * i], pts[3LL * i + 1], pts[3LL * i + 2]);
        p->setOptFixed(pfix[i] != 0);
        points.push_back(p);
    }
    for (int k = 0; k < no; ++k) {
        cv::KeyPoint kp;
        kp.pt = cv::Point2f((float)uv[2LL * k], (float)uv[2LL * k + 1]);
        auto o = std::make_shared<OB::KeyPoint2D>(kp, cv::Mat());
        o->setPointUd(cv::Point2f((float)uv[2LL * k], (float)uv[2LL * k + 1]));
        o->setFrame(frames[oc[k]]);
        o->setWorldObject(points[op[k]]);
        points[op[k]]->addObservation(o);
        frame_obs[oc[k]].push_back(o);
    }
    for (int c = 0; c < nc; ++c) frames[c]->setObservations(frame_obs[c]);

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
        const auto T = frames[c]->getPose()->getPose();
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 4; ++j) {
                const double v = T(i, j);
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
