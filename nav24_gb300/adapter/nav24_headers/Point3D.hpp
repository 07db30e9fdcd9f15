// Stand-in for core/scene/worldObject/Point3D.hpp:12-28.
#pragma once
#include <opencv2/core.hpp>
#include "WorldObject.hpp"
namespace NAV24::WO {
class Point3D : public WorldObject {
public:
    Point3D(double x, double y, double z) : mPoint(x, y, z) {}
    [[nodiscard]] const cv::Point3d& getPoint() const { return mPoint; }
    void setPoint(const cv::Point3d& p) { mPoint = p; }
protected:
    cv::Point3d mPoint;
};
}  // namespace NAV24::WO
