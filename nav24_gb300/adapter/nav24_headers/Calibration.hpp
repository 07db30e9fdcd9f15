// Stand-in for core/sensor/camera/Calibration.hpp:21-55 (pinhole intrinsics only: getK_ei).
#pragma once
#include <memory>
#include <eigen3/Eigen/Dense>
namespace NAV24 {
class Calibration {
public:
    Calibration(float fx, float fy, float cx, float cy) {
        K = Eigen::Matrix3f::Identity();
        K(0, 0) = fx; K(1, 1) = fy; K(0, 2) = cx; K(1, 2) = cy;
    }
    Eigen::Matrix3f getK_ei() { return K; }
protected:
    Eigen::Matrix3f K;
};
typedef std::shared_ptr<Calibration> CalibPtr;
}  // namespace NAV24
