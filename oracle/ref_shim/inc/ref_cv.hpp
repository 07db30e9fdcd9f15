// ref_cv.hpp - stand-in for the part of OpenCV's core API that nav24's camera-model, calibration,
// parameter and observation sources name (TEST INFRASTRUCTURE: only the reference-pin recipe,
// oracle/ref_build.py, compiles against it).  OpenCV is not installed here.
//
// Provided with a working implementation (what the reference-pin harness exercises): the point,
// rectangle and keypoint types; Mat holding CV_32F or CV_64F elements with eye/zeros, clone,
// ptr, at, empty, the Mat_ comma initializer and printing.  Declared so the sources compile, but
// not exercised (they end the process if reached): Mat products, transpose, inverse and the
// undistortion routines of calib3d.
#pragma once

#include <cassert>  // the real library headers pull it in; nav24 relies on that
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>  // like assert, pulled in by the real headers
#include <memory>
#include <sstream>
#include <string>
#include <vector>

#define CV_8U 0
#define CV_32F 5
#define CV_64F 6
#define CV_PI 3.1415926535897932384626433832795

namespace cv {

[[noreturn]] inline void ref_cv_unavailable(const char* what) {
    std::fprintf(stderr, "OpenCV stand-in: %s is not provided\n", what);
    std::abort();
}

template <class T>
struct Point_ {
    T x, y;
    Point_() : x(0), y(0) {}
    Point_(T x_, T y_) : x(x_), y(y_) {}
    template <class U>
    operator Point_<U>() const {
        return Point_<U>(static_cast<U>(x), static_cast<U>(y));
    }
};
typedef Point_<float> Point2f;
typedef Point_<double> Point2d;
typedef Point_<int> Point;

template <class T>
struct Point3_ {
    T x, y, z;
    Point3_() : x(0), y(0), z(0) {}
    Point3_(T x_, T y_, T z_) : x(x_), y(y_), z(z_) {}
    template <class U>
    operator Point3_<U>() const {
        return Point3_<U>(static_cast<U>(x), static_cast<U>(y), static_cast<U>(z));
    }
};
typedef Point3_<float> Point3f;
typedef Point3_<double> Point3d;

template <class T>
struct Rect_ {
    T x, y, width, height;
    Rect_() : x(0), y(0), width(0), height(0) {}
    Rect_(T x_, T y_, T w_, T h_) : x(x_), y(y_), width(w_), height(h_) {}
};
typedef Rect_<float> Rect2f;

struct KeyPoint {
    Point2f pt;
    float size = 0.f, angle = -1.f, response = 0.f;
    int octave = 0, class_id = -1;
    KeyPoint() = default;
};

// Dense 2-D matrix of 8-bit, FP32 or FP64 elements; copies share the data, clone() does not.
class Mat {
public:
    int rows = 0, cols = 0;

    Mat() = default;
    Mat(int r, int c, int type) : rows(r), cols(c), type_(type) {
        data_ = std::make_shared<std::vector<unsigned char>>((size_t)r * c * elem_size(type), 0);
    }

    static Mat zeros(int r, int c, int type) { return Mat(r, c, type); }
    static Mat eye(int r, int c, int type) {
        Mat m(r, c, type);
        for (int k = 0; k < (r < c ? r : c); ++k) m.set(k, k, 1.0);
        return m;
    }

    int type() const { return type_; }
    bool empty() const { return !data_ || rows * cols == 0; }
    Mat clone() const {
        Mat m;
        m.rows = rows;
        m.cols = cols;
        m.type_ = type_;
        if (data_) m.data_ = std::make_shared<std::vector<unsigned char>>(*data_);
        return m;
    }

    template <class T>
    T* ptr(int r = 0) {
        return reinterpret_cast<T*>(data_->data()) + (size_t)r * cols;
    }
    template <class T>
    const T* ptr(int r = 0) const {
        return reinterpret_cast<const T*>(data_->data()) + (size_t)r * cols;
    }
    template <class T>
    T& at(int r, int c) {
        return ptr<T>()[(size_t)r * cols + c];
    }
    template <class T>
    const T& at(int r, int c) const {
        return ptr<T>()[(size_t)r * cols + c];
    }
    template <class T>
    T& at(int k) {
        return ptr<T>()[k];
    }
    template <class T>
    const T& at(int k) const {
        return ptr<T>()[k];
    }

    double get(int r, int c) const {
        if (type_ == CV_32F) return at<float>(r, c);
        if (type_ == CV_64F) return at<double>(r, c);
        return at<unsigned char>(r, c);
    }
    void set(int r, int c, double v) {
        if (type_ == CV_32F) at<float>(r, c) = static_cast<float>(v);
        else if (type_ == CV_64F) at<double>(r, c) = v;
        else at<unsigned char>(r, c) = static_cast<unsigned char>(v);
    }

    Mat t() const { ref_cv_unavailable("Mat::t"); }
    Mat inv() const { ref_cv_unavailable("Mat::inv"); }
    Mat row(int) const { ref_cv_unavailable("Mat::row"); }
    friend Mat operator*(const Mat&, const Mat&) { ref_cv_unavailable("Mat product"); }
    friend Mat operator-(const Mat&) { ref_cv_unavailable("Mat negation"); }

private:
    static size_t elem_size(int type) { return type == CV_64F ? 8 : type == CV_32F ? 4 : 1; }
    int type_ = CV_8U;
    std::shared_ptr<std::vector<unsigned char>> data_;
};

inline std::ostream& operator<<(std::ostream& os, const Mat& m) {
    os << "[";
    for (int r = 0; r < m.rows; ++r)
        for (int c = 0; c < m.cols; ++c) os << (c ? ", " : (r ? ";\n " : "")) << m.get(r, c);
    return os << "]";
}

template <class T>
struct DataType;
template <>
struct DataType<float> {
    static constexpr int type = CV_32F;
};
template <>
struct DataType<double> {
    static constexpr int type = CV_64F;
};

// `Mat_<T>(r, c) << a, b, ...` fills row by row and converts to Mat.
template <class T>
class MatCommaInitializer_ {
public:
    MatCommaInitializer_(const Mat& m, int k) : m_(m), k_(k) {}
    template <class V>
    MatCommaInitializer_& operator,(const V& v) {
        m_.at<T>(k_ / m_.cols, k_ % m_.cols) = static_cast<T>(v);
        ++k_;
        return *this;
    }
    operator Mat() const { return m_; }

private:
    Mat m_;
    int k_;
};

template <class T>
class Mat_ : public Mat {
public:
    Mat_(int r, int c) : Mat(r, c, DataType<T>::type) {}
    template <class V>
    MatCommaInitializer_<T> operator<<(const V& v) {
        at<T>(0, 0) = static_cast<T>(v);
        return MatCommaInitializer_<T>(*this, 1);
    }
};

template <class A, class B, class C, class D, class E, class F>
void undistortPoints(const A&, B&, const C&, const D&, const E&, const F&) {
    ref_cv_unavailable("undistortPoints");
}

namespace fisheye {
template <class A, class B, class C, class D, class E, class F>
void undistortPoints(const A&, B&, const C&, const D&, const E&, const F&) {
    ref_cv_unavailable("fisheye::undistortPoints");
}
}  // namespace fisheye

}  // namespace cv
