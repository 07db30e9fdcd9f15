// ref_eigen.hpp - stand-in for the fixed-size part of Eigen 3 that nav24's edge and camera-model
// sources use (TEST INFRASTRUCTURE: only the reference-pin recipe, oracle/ref_build.py, compiles
// against it).  Eigen is not installed here; this header provides the same names and signatures
// with a small dense implementation of its own:
//   Matrix<T, R, C> (column-major storage, as Eigen's default), the comma initializer (row by row),
//   (), [], unary and binary +/-, matrix products (sum over k in increasing order), scalar
//   products, transpose, cast, Zero/Identity; the Vector/Matrix typedefs; Quaternion<T> with
//   toRotationMatrix, the rotation of a vector and construction from a rotation matrix.
// Results agree with Eigen's to rounding (Eigen may sum small products in another order or
// with SIMD); the parity tests that use the reference build allow 1e-12 relative.
#pragma once

#include <cassert>  // the real library headers pull it in; nav24 relies on that
#include <cmath>
#include <cstddef>
#include <ostream>

#define EIGEN_MAKE_ALIGNED_OPERATOR_NEW
#define EIGEN_WORLD_VERSION 3
#define EIGEN_MAJOR_VERSION 4
#define EIGEN_MINOR_VERSION 0

namespace Eigen {

template <class T, int R, int C>
class Matrix;

// Fills a matrix in row-major order from `m << a, b, c, ...`.
template <class M>
class CommaInitializer {
public:
    CommaInitializer(M& m, int k) : m_(m), k_(k) {}
    template <class V>
    CommaInitializer& operator,(const V& v) {
        m_.row_major(k_++) = static_cast<typename M::Scalar>(v);
        return *this;
    }

private:
    M& m_;
    int k_;
};

template <class T, int R, int C>
class Matrix {
public:
    using Scalar = T;
    static constexpr int RowsAtCompileTime = R;
    static constexpr int ColsAtCompileTime = C;

    Matrix() {
        for (int k = 0; k < R * C; ++k) d_[k] = T(0);
    }
    Matrix(T a, T b) {  // 2-vectors
        static_assert(R * C == 2, "two-value constructor of a 2-vector");
        d_[0] = a;
        d_[1] = b;
    }
    Matrix(T a, T b, T c) {  // 3-vectors
        static_assert(R * C == 3, "three-value constructor of a 3-vector");
        d_[0] = a;
        d_[1] = b;
        d_[2] = c;
    }

    static Matrix Zero() { return Matrix(); }
    static Matrix Identity() {
        Matrix m;
        for (int k = 0; k < (R < C ? R : C); ++k) m(k, k) = T(1);
        return m;
    }

    int rows() const { return R; }
    int cols() const { return C; }
    int size() const { return R * C; }

    T& operator()(int i, int j) { return d_[i + R * j]; }
    const T& operator()(int i, int j) const { return d_[i + R * j]; }
    T& operator()(int k) { return d_[k]; }
    const T& operator()(int k) const { return d_[k]; }
    T& operator[](int k) { return d_[k]; }
    const T& operator[](int k) const { return d_[k]; }
    T& row_major(int k) { return (*this)(k / C, k % C); }

    T& x() { return d_[0]; }
    T& y() { return d_[1]; }
    T& z() { return d_[2]; }
    const T& x() const { return d_[0]; }
    const T& y() const { return d_[1]; }
    const T& z() const { return d_[2]; }

    T* data() { return d_; }
    const T* data() const { return d_; }

    template <class V>
    CommaInitializer<Matrix> operator<<(const V& v) {
        row_major(0) = static_cast<T>(v);
        return CommaInitializer<Matrix>(*this, 1);
    }

    Matrix operator-() const {
        Matrix m;
        for (int k = 0; k < R * C; ++k) m.d_[k] = -d_[k];
        return m;
    }
    Matrix& operator+=(const Matrix& o) {
        for (int k = 0; k < R * C; ++k) d_[k] += o.d_[k];
        return *this;
    }
    Matrix& operator-=(const Matrix& o) {
        for (int k = 0; k < R * C; ++k) d_[k] -= o.d_[k];
        return *this;
    }
    friend Matrix operator+(const Matrix& a, const Matrix& b) {
        Matrix m = a;
        m += b;
        return m;
    }
    friend Matrix operator-(const Matrix& a, const Matrix& b) {
        Matrix m = a;
        m -= b;
        return m;
    }
    friend Matrix operator*(const Matrix& a, T s) {
        Matrix m;
        for (int k = 0; k < R * C; ++k) m.d_[k] = a.d_[k] * s;
        return m;
    }
    friend Matrix operator*(T s, const Matrix& a) { return a * s; }
    friend Matrix operator/(const Matrix& a, T s) {
        Matrix m;
        for (int k = 0; k < R * C; ++k) m.d_[k] = a.d_[k] / s;
        return m;
    }

    template <int K>
    Matrix<T, R, K> operator*(const Matrix<T, C, K>& b) const {
        Matrix<T, R, K> m;
        for (int i = 0; i < R; ++i)
            for (int j = 0; j < K; ++j) {
                T s = (*this)(i, 0) * b(0, j);
                for (int k = 1; k < C; ++k) s += (*this)(i, k) * b(k, j);
                m(i, j) = s;
            }
        return m;
    }

    Matrix<T, C, R> transpose() const {
        Matrix<T, C, R> m;
        for (int i = 0; i < R; ++i)
            for (int j = 0; j < C; ++j) m(j, i) = (*this)(i, j);
        return m;
    }

    template <class U>
    Matrix<U, R, C> cast() const {
        Matrix<U, R, C> m;
        for (int k = 0; k < R * C; ++k) m[k] = static_cast<U>(d_[k]);
        return m;
    }

    T squaredNorm() const {
        T s = T(0);
        for (int k = 0; k < R * C; ++k) s += d_[k] * d_[k];
        return s;
    }
    T norm() const { return std::sqrt(squaredNorm()); }
    T dot(const Matrix& o) const {
        T s = T(0);
        for (int k = 0; k < R * C; ++k) s += d_[k] * o.d_[k];
        return s;
    }
    Matrix cross(const Matrix& o) const {
        static_assert(R * C == 3, "cross product of 3-vectors");
        return Matrix(d_[1] * o.d_[2] - d_[2] * o.d_[1], d_[2] * o.d_[0] - d_[0] * o.d_[2],
                      d_[0] * o.d_[1] - d_[1] * o.d_[0]);
    }

private:
    T d_[R * C];
};

template <class T, int R, int C>
std::ostream& operator<<(std::ostream& os, const Matrix<T, R, C>& m) {
    for (int i = 0; i < R; ++i) {
        for (int j = 0; j < C; ++j) os << (j ? " " : "") << m(i, j);
        if (i + 1 < R) os << "\n";
    }
    return os;
}

typedef Matrix<double, 2, 1> Vector2d;
typedef Matrix<double, 3, 1> Vector3d;
typedef Matrix<double, 4, 1> Vector4d;
typedef Matrix<double, 6, 1> Vector6d;
typedef Matrix<float, 2, 1> Vector2f;
typedef Matrix<float, 3, 1> Vector3f;
typedef Matrix<double, 2, 2> Matrix2d;
typedef Matrix<double, 3, 3> Matrix3d;
typedef Matrix<double, 4, 4> Matrix4d;
typedef Matrix<float, 3, 3> Matrix3f;
typedef Matrix<float, 4, 4> Matrix4f;

// Unit quaternion (w, x, y, z) acting on 3-vectors.
template <class T>
class Quaternion {
public:
    Quaternion() : w_(T(1)), x_(T(0)), y_(T(0)), z_(T(0)) {}
    Quaternion(T w, T x, T y, T z) : w_(w), x_(x), y_(y), z_(z) {}
    // From a rotation matrix: the trace when positive, else the largest diagonal entry
    // (Shepperd, J. Guidance & Control 1978).
    explicit Quaternion(const Matrix<T, 3, 3>& m) {
        const T tr = m(0, 0) + m(1, 1) + m(2, 2);
        if (tr > T(0)) {
            T s = std::sqrt(tr + T(1));
            w_ = T(0.5) * s;
            s = T(0.5) / s;
            x_ = (m(2, 1) - m(1, 2)) * s;
            y_ = (m(0, 2) - m(2, 0)) * s;
            z_ = (m(1, 0) - m(0, 1)) * s;
        } else {
            int i = 0;
            if (m(1, 1) > m(0, 0)) i = 1;
            if (m(2, 2) > m(i, i)) i = 2;
            const int j = (i + 1) % 3, k = (j + 1) % 3;
            T v[3];
            T s = std::sqrt(m(i, i) - m(j, j) - m(k, k) + T(1));
            v[i] = T(0.5) * s;
            s = T(0.5) / s;
            w_ = (m(k, j) - m(j, k)) * s;
            v[j] = (m(j, i) + m(i, j)) * s;
            v[k] = (m(k, i) + m(i, k)) * s;
            x_ = v[0];
            y_ = v[1];
            z_ = v[2];
        }
    }

    T& w() { return w_; }
    T& x() { return x_; }
    T& y() { return y_; }
    T& z() { return z_; }
    const T& w() const { return w_; }
    const T& x() const { return x_; }
    const T& y() const { return y_; }
    const T& z() const { return z_; }

    T norm() const { return std::sqrt(w_ * w_ + x_ * x_ + y_ * y_ + z_ * z_); }
    void normalize() {
        const T n = norm();
        w_ /= n;
        x_ /= n;
        y_ /= n;
        z_ /= n;
    }
    Quaternion normalized() const {
        Quaternion q = *this;
        q.normalize();
        return q;
    }
    Quaternion conjugate() const { return Quaternion(w_, -x_, -y_, -z_); }
    Quaternion inverse() const {
        const T n2 = w_ * w_ + x_ * x_ + y_ * y_ + z_ * z_;
        return Quaternion(w_ / n2, -x_ / n2, -y_ / n2, -z_ / n2);
    }

    Matrix<T, 3, 3> toRotationMatrix() const {
        const T tx = T(2) * x_, ty = T(2) * y_, tz = T(2) * z_;
        const T twx = tx * w_, twy = ty * w_, twz = tz * w_;
        const T txx = tx * x_, txy = ty * x_, txz = tz * x_;
        const T tyy = ty * y_, tyz = tz * y_, tzz = tz * z_;
        Matrix<T, 3, 3> r;
        r(0, 0) = T(1) - (tyy + tzz);
        r(0, 1) = txy - twz;
        r(0, 2) = txz + twy;
        r(1, 0) = txy + twz;
        r(1, 1) = T(1) - (txx + tzz);
        r(1, 2) = tyz - twx;
        r(2, 0) = txz - twy;
        r(2, 1) = tyz + twx;
        r(2, 2) = T(1) - (txx + tyy);
        return r;
    }

    // v' = q v q^-1 written as v + w t + u x t with t = 2 u x v (u the vector part).
    Matrix<T, 3, 1> operator*(const Matrix<T, 3, 1>& v) const {
        const Matrix<T, 3, 1> u(x_, y_, z_);
        Matrix<T, 3, 1> t = u.cross(v);
        t = t * T(2);
        return v + t * w_ + u.cross(t);
    }

    Quaternion operator*(const Quaternion& b) const {
        return Quaternion(w_ * b.w_ - x_ * b.x_ - y_ * b.y_ - z_ * b.z_,
                          w_ * b.x_ + x_ * b.w_ + y_ * b.z_ - z_ * b.y_,
                          w_ * b.y_ + y_ * b.w_ + z_ * b.x_ - x_ * b.z_,
                          w_ * b.z_ + z_ * b.w_ + x_ * b.y_ - y_ * b.x_);
    }

private:
    T w_, x_, y_, z_;
};

typedef Quaternion<double> Quaterniond;
typedef Quaternion<float> Quaternionf;

}  // namespace Eigen
