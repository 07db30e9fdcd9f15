// Stand-in for the OpenCV point types nav24's data model exposes (cv::Point2f, cv::Point3f,
// cv::Point3d, cv::KeyPoint, cv::Mat as an opaque type).
#pragma once
namespace cv {
template <class T>
struct Point_ {
    T x = 0, y = 0;
    Point_() = default;
    Point_(T x_, T y_) : x(x_), y(y_) {}
};
template <class T>
struct Point3_ {
    T x = 0, y = 0, z = 0;
    Point3_() = default;
    Point3_(T x_, T y_, T z_) : x(x_), y(y_), z(z_) {}
    template <class U>
    operator Point3_<U>() const { return Point3_<U>((U)x, (U)y, (U)z); }
};
using Point2f = Point_<float>;
using Point3f = Point3_<float>;
using Point3d = Point3_<double>;
struct KeyPoint {
    Point2f pt;
};
struct Mat {};
}  // namespace cv
