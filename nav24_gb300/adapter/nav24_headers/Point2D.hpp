// Stand-in for core/sensorData/observation/Point2D.hpp:17-77 (Point2D, KeyPoint2D).
#pragma once
#include <opencv2/core.hpp>
#include "Observation.hpp"
namespace NAV24::OB {
class Point2D : public Observation {
public:
    Point2D(float x, float y) : mPoint(x, y) {}
    cv::Point2f getPoint() { return mPoint; }
    cv::Point2f getPointUd() { return mPointUd; }
    void setPointUd(const cv::Point2f& p) { mPointUd = p; }
protected:
    cv::Point2f mPoint, mPointUd;
};
class KeyPoint2D : public Point2D {
public:
    KeyPoint2D(cv::KeyPoint kpt, const cv::Mat&) : Point2D(kpt.pt.x, kpt.pt.y), mKPt(kpt) {}
    [[nodiscard]] const cv::KeyPoint& getKeyPoint() const { return mKPt; }
protected:
    cv::KeyPoint mKPt;
};
}  // namespace NAV24::OB
