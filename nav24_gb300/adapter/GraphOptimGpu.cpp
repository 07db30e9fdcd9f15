// GraphOptimGpu.cpp - see GraphOptimGpu.hpp.
//
// The flattening follows nav24's graph build (core/backEnd/BE_GraphOptim.cpp):
//  * addFrameVertices (:79-100): one pose vertex per frame with a pose, ids 0.. in frame order,
//    fixed from Frame::isOptFixed, Frame::setOptId(id);
//  * extractMapPoints (:102-115): the world objects seen by the frames' observations;
//  * addMapPointVertices (:117-211): Point3D objects that are valid, initial estimate rounded to
//    float (Converter::toVector3d(cv::Point3f), :147), fixed from isOptFixed; one edge per
//    observation of the point that is valid, has a frame whose optId names a pose vertex, and is a
//    KeyPoint2D; measurement getPointUd() (float); a point with no edge is dropped (:204-205);
//    Huber with delta float(sqrt(5.99)) when PR_VBA::mbRobust (:125, :191-195);
//  * nothing is done (and optIds stay as set) when there is no pose or no point vertex (:59-63);
//  * recoverPose (:213-229): every pose vertex's frame gets a new PoseSE3 (ref, target and
//    timestamp of its previous pose) and optId -1; recoverMapPoints (:231-243): every point vertex
//    gets its optimized position rounded to float.
// Points are taken in first-seen order; nav24's std::set orders them by heap address, which only
// changes the floating-point summation order.
#include "GraphOptimGpu.hpp"

#include <cmath>
#include <cstring>
#include <unordered_map>

#include "Calibration.hpp"
#include "Frame.hpp"
#include "Point2D.hpp"
#include "Point3D.hpp"

namespace NAV24::BE {

struct GraphOptimGpu::Flat {
    std::vector<FramePtr> frames;             // pose vertices, id order
    std::vector<std::shared_ptr<WO::Point3D>> points;  // point vertices with >= 1 edge
    std::vector<double> cam_pose, pts, uv;
    std::vector<uint8_t> cam_fixed, pt_fixed;
    std::vector<int32_t> obs_cam, obs_pt;
    double intr[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    int iterations = 5;
    bool robust = false;
    std::vector<double> pose_out, pts_out, trace;
    nav_ba_problem prob{};
};

GraphOptimGpu::GraphOptimGpu(int device, int precision) {
    nav_ba_options_default(&options);
    options.precision = precision;
    mStatus = nav_ba_create(&mCtx, device);
}

GraphOptimGpu::~GraphOptimGpu() { nav_ba_destroy(mCtx); }

const char* GraphOptimGpu::lastError() const { return mCtx ? nav_ba_last_error(mCtx) : "no CUDA device"; }

bool GraphOptimGpu::flatten(const ProblemPtr& problem, Flat& f) {
    auto pProblem = std::dynamic_pointer_cast<PR_VBA>(problem);
    if (!pProblem) return false;
    f.iterations = problem->getNumIter();
    f.robust = pProblem->mbRobust;
    if (pProblem->mpCalib) {
        const auto K = pProblem->mpCalib->getK_ei();  // float intrinsics (GeometricCamera.h:117)
        f.intr[0] = K(0, 0);
        f.intr[1] = K(1, 1);
        f.intr[2] = K(0, 2);
        f.intr[3] = K(1, 2);
    }
    // pose vertices
    for (const auto& pFrame : pProblem->mvpFrames) {
        if (!pFrame || !pFrame->getPose()) continue;
        const unsigned long id = f.frames.size();
        const auto T = pFrame->getPose()->getPose();
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 4; ++c) f.cam_pose.push_back(T(r, c));
        f.cam_fixed.push_back(pFrame->isOptFixed() ? 1 : 0);
        pFrame->setOptId(id);
        f.frames.push_back(pFrame);
    }
    const unsigned long n_pose = f.frames.size();
    // map points seen by the frames (first-seen order)
    std::vector<WO::WoPtr> seen;
    std::unordered_map<const WO::WorldObject*, int> seen_idx;
    for (const auto& pFrame : pProblem->mvpFrames) {
        if (!pFrame) continue;
        for (const auto& pObs : pFrame->getObservations()) {
            if (!pObs) continue;
            auto pWo = pObs->getWorldObject();
            if (pWo && seen_idx.emplace(pWo.get(), (int)seen.size()).second) seen.push_back(pWo);
        }
    }
    for (const auto& pWo : seen) {
        auto pPt = std::dynamic_pointer_cast<WO::Point3D>(pWo);
        if (!pPt || !pPt->isValid()) continue;
        const int32_t pid = (int32_t)f.points.size();
        int n_edges = 0;
        for (const auto& wObs : pWo->getObservations()) {
            auto pObs = wObs.lock();
            if (!pObs || !pObs->isValid() || !pObs->getFrame()) continue;
            const unsigned long frameId = pObs->getFrame()->getOptId();
            if (frameId >= n_pose) continue;  // not a pose vertex of this problem
            auto pKp = std::dynamic_pointer_cast<OB::KeyPoint2D>(pObs);
            if (!pKp) continue;
            const cv::Point2f z = pKp->getPointUd();
            f.uv.push_back(z.x);
            f.uv.push_back(z.y);
            f.obs_cam.push_back((int32_t)frameId);
            f.obs_pt.push_back(pid);
            ++n_edges;
        }
        if (n_edges == 0) continue;
        const cv::Point3f p32 = pPt->getPoint();  // float rounding of the initial estimate
        f.pts.push_back(p32.x);
        f.pts.push_back(p32.y);
        f.pts.push_back(p32.z);
        f.pt_fixed.push_back(pPt->isOptFixed() ? 1 : 0);
        f.points.push_back(pPt);
    }
    f.prob.n_cams = (int32_t)f.frames.size();
    f.prob.n_points = (int32_t)f.points.size();
    f.prob.n_obs = (int32_t)f.obs_cam.size();
    f.prob.cam_pose = f.cam_pose.data();
    f.prob.cam_fixed = f.cam_fixed.data();
    f.prob.points = f.pts.data();
    f.prob.point_fixed = f.pt_fixed.data();
    f.prob.obs_uv = f.uv.data();
    f.prob.obs_cam = f.obs_cam.data();
    f.prob.obs_point = f.obs_pt.data();
    f.prob.camera_model = NAV_BA_CAM_PINHOLE;
    std::memcpy(f.prob.intrinsics, f.intr, sizeof(f.intr));
    f.pose_out.assign(12 * f.frames.size(), 0.0);
    f.pts_out.assign(3 * f.points.size(), 0.0);
    f.trace.assign(f.iterations + 1, 0.0);
    return !f.frames.empty() && !f.points.empty();
}

void GraphOptimGpu::recover(Flat& f, const nav_ba_result& r) {
    (void)r;
    for (size_t c = 0; c < f.frames.size(); ++c) {
        const auto& pFrame = f.frames[c];
        auto pLast = pFrame->getPose();
        Eigen::Matrix4d T = Eigen::Matrix4d::Identity();
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 4; ++j) T(i, j) = f.pose_out[12 * c + 4 * i + j];
        pFrame->setPose(std::make_shared<TF::PoseSE3>(pLast->getRef(), pLast->getTarget(), pLast->getTimestamp(), T));
        pFrame->setOptId((unsigned long)-1);
    }
    for (size_t k = 0; k < f.points.size(); ++k) {
        const cv::Point3f p((float)f.pts_out[3 * k], (float)f.pts_out[3 * k + 1], (float)f.pts_out[3 * k + 2]);
        f.points[k]->setPoint(p);
    }
}

void GraphOptimGpu::solve(const ProblemPtr& problem) {
    solveBatched({problem});
}

void GraphOptimGpu::solveBatched(const std::vector<ProblemPtr>& problems) {
    mResults.clear();
    if (!mCtx) {
        mStatus = NAV_BA_ERR_NO_DEVICE;
        return;
    }
    std::vector<Flat> flats(problems.size());
    std::vector<int> solvable;
    for (size_t i = 0; i < problems.size(); ++i)
        if (flatten(problems[i], flats[i])) solvable.push_back((int)i);
    mResults.assign(problems.size(), nav_ba_result{});
    mStatus = NAV_BA_OK;
    if (solvable.empty()) {
        mStatus = NAV_BA_EMPTY;  // nav24 logs "ill-conditioned" and returns (BE_GraphOptim.cpp:59-63)
        return;
    }
    // windows that share iterations / robust settings go in one call
    size_t i0 = 0;
    while (i0 < solvable.size()) {
        const Flat& f0 = flats[solvable[i0]];
        size_t i1 = i0 + 1;
        while (i1 < solvable.size() && flats[solvable[i1]].iterations == f0.iterations &&
               flats[solvable[i1]].robust == f0.robust &&
               std::memcmp(flats[solvable[i1]].intr, f0.intr, sizeof(f0.intr)) == 0)
            ++i1;
        nav_ba_options o = options;
        o.iterations = f0.iterations;
        o.robust = f0.robust ? 1 : 0;
        o.huber_delta = (double)(float)std::sqrt(5.99);
        std::vector<nav_ba_problem> probs;
        std::vector<nav_ba_result> res;
        for (size_t k = i0; k < i1; ++k) {
            Flat& f = flats[solvable[k]];
            probs.push_back(f.prob);
            nav_ba_result r{};
            r.cam_pose_out = f.pose_out.data();
            r.points_out = f.pts_out.data();
            r.cost_trace = f.trace.data();
            res.push_back(r);
        }
        const nav_ba_status st = nav_ba_solve_batched(mCtx, probs.data(), (int32_t)probs.size(), &o, res.data());
        if (st != NAV_BA_OK) {
            mStatus = st;  // nothing written back, like an optimizer that failed to run
            return;
        }
        for (size_t k = i0; k < i1; ++k) {
            const nav_ba_result& r = res[k - i0];
            mResults[solvable[k]] = r;
            if (r.status == NAV_BA_OK) recover(flats[solvable[k]], r);
        }
        i0 = i1;
    }
}

}  // namespace NAV24::BE
