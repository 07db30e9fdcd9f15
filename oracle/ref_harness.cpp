// ref_harness.cpp - C entry points over nav24's own edge and camera-model code (TEST
// INFRASTRUCTURE).  oracle/ref_build.py compiles this file together with the reference's
// unmodified sources, read where they lie in the reference tree:
//   core/dataTypes/optimization/OptimizableTypes.cpp   EdgeSE3ProjectXYZ (computeError and
//                                                       isDepthPositive are inline in the .hpp)
//   core/sensor/camera/Calibration.cpp                 Calibration::getCalibParams, loadParams,
//                                                       project, projectJac
//   core/sensor/camera/models/{Pinhole,PinholeRadTan,KannalaBrandt8}.cpp
//   core/tools/parameters/Parameter.cpp, core/sensorData/observation/Point2D.cpp,
//   core/scene/worldObject/{Point3D,WorldObject}.cpp   (what Calibration.cpp links against)
// and stand-in headers for Eigen, OpenCV, Boost.Serialization, glog and g2o (oracle/ref_shim),
// which are absent here.  The output library goes to oracle/_ref/ and is loaded only by the tests
// that pin the oracle and the GPU path to the reference's own arithmetic.
#include <cstdint>
#include <memory>
#include <string>
#include <vector>

#include "Calibration.hpp"
#include "OptimizableTypes.hpp"
#include "Parameter.hpp"

#include "../include/nav_ba.h"

namespace {

// The calibration object nav24 builds for the problem's camera: intrinsics and distortion go
// through Calibration::getCalibParams (K and D as CV_64F matrices, as the calibration front end
// passes them) and Calibration's constructor, which rounds every parameter to float
// (Calibration.cpp:42-60) and picks the model by distType (:78-87).
std::shared_ptr<NAV24::Calibration> make_calibration(const nav_ba_problem& p,
                                                     std::vector<NAV24::ParamPtr>& holder) {
    cv::Mat K = cv::Mat::eye(3, 3, CV_64F);
    K.at<double>(0, 0) = p.intrinsics[0];
    K.at<double>(1, 1) = p.intrinsics[1];
    K.at<double>(0, 2) = p.intrinsics[2];
    K.at<double>(1, 2) = p.intrinsics[3];
    std::string dist_type;
    cv::Mat D;
    if (p.camera_model == NAV_BA_CAM_KANNALA_BRANDT8) {
        dist_type = "kannala-brandt8";
        D = cv::Mat::zeros(4, 1, CV_64F);
        for (int k = 0; k < 4; ++k) D.at<double>(k, 0) = p.intrinsics[4 + k];
    }
    NAV24::ParamPtr root = NAV24::Calibration::getCalibParams(K, D, dist_type, holder);
    return std::make_shared<NAV24::Calibration>(root);
}

}  // namespace

extern "C" {

// Residual, Jacobians and depth test of every observation of `p` at its given state, computed by
// nav24's EdgeSE3ProjectXYZ exactly as GraphOptim sets it up (BE_GraphOptim.cpp:91-93,146-197):
// pose vertex estimate SE3Quat(R, t) of T_cw, point vertex estimate, measurement, pCamera.
//   e [n_obs][2], jc [n_obs][2][6] (_jacobianOplusXj, the pose), jp [n_obs][2][3]
//   (_jacobianOplusXi, the point), depth_positive [n_obs] (isDepthPositive); any may be NULL.
// Pinhole and Kannala-Brandt 8 models only (the radial model has no reference counterpart).
int32_t ref_edges(const nav_ba_problem* p, double* e, double* jc, double* jp, uint8_t* depth_positive) {
    if (!p || (p->camera_model != NAV_BA_CAM_PINHOLE && p->camera_model != NAV_BA_CAM_KANNALA_BRANDT8))
        return NAV_BA_ERR_ARGUMENT;
    std::vector<NAV24::ParamPtr> holder;
    const std::shared_ptr<NAV24::Calibration> calib = make_calibration(*p, holder);
    for (int32_t k = 0; k < p->n_obs; ++k) {
        const double* T = p->cam_pose + 12LL * p->obs_cam[k];
        Eigen::Matrix3d R;
        R << T[0], T[1], T[2], T[4], T[5], T[6], T[8], T[9], T[10];
        const Eigen::Vector3d t(T[3], T[7], T[11]);
        const double* X = p->points + 3LL * p->obs_point[k];
        ORB_SLAM3::MyVertexSE3Expmap pose;
        pose.setEstimate(g2o::SE3Quat(R, t));
        ORB_SLAM3::MyVertexSBAPointXYZ point;
        point.setEstimate(Eigen::Vector3d(X[0], X[1], X[2]));
        ORB_SLAM3::EdgeSE3ProjectXYZ edge;
        edge.setVertex(0, &point);
        edge.setVertex(1, &pose);
        edge.setMeasurement(Eigen::Vector2d(p->obs_uv[2LL * k], p->obs_uv[2LL * k + 1]));
        edge.pCamera = calib;
        edge.computeError();
        if (e) {
            e[2LL * k] = edge.error()[0];
            e[2LL * k + 1] = edge.error()[1];
        }
        if (depth_positive) depth_positive[k] = edge.isDepthPositive() ? 1 : 0;
        if (jc || jp) {
            edge.linearizeOplus();
            for (int r = 0; r < 2; ++r) {
                if (jp)
                    for (int c = 0; c < 3; ++c) jp[6LL * k + 3 * r + c] = edge.jacobianOplusXi()(r, c);
                if (jc)
                    for (int c = 0; c < 6; ++c) jc[12LL * k + 6 * r + c] = edge.jacobianOplusXj()(r, c);
            }
        }
    }
    return NAV_BA_OK;
}

// The camera model's own project / projectJac through Calibration (Calibration.cpp:235-247):
// uv [n][2] and jac [n][2][3] of the camera-frame points xc [n][3]; either output may be NULL.
int32_t ref_project(const nav_ba_problem* p, int32_t n, const double* xc, double* uv, double* jac) {
    if (!p || n < 0 || (n && !xc)) return NAV_BA_ERR_ARGUMENT;
    std::vector<NAV24::ParamPtr> holder;
    const std::shared_ptr<NAV24::Calibration> calib = make_calibration(*p, holder);
    for (int32_t k = 0; k < n; ++k) {
        const Eigen::Vector3d x(xc[3LL * k], xc[3LL * k + 1], xc[3LL * k + 2]);
        if (uv) {
            const Eigen::Vector2d u = calib->project(x);
            uv[2LL * k] = u[0];
            uv[2LL * k + 1] = u[1];
        }
        if (jac) {
            const Eigen::Matrix<double, 2, 3> J = calib->projectJac(x);
            for (int r = 0; r < 2; ++r)
                for (int c = 0; c < 3; ++c) jac[6LL * k + 3 * r + c] = J(r, c);
        }
    }
    return NAV_BA_OK;
}

}  // extern "C"
