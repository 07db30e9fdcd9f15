// ref_g2o.hpp - stand-in for the g2o names that nav24's EdgeSE3ProjectXYZ and its vertex subclasses
// use (TEST INFRASTRUCTURE: only the reference-pin recipe, oracle/ref_build.py, compiles against
// it).  g2o is not vendored by the reference and not installed here.
//
// What the reference-pin harness exercises is the reference's own edge code (computeError,
// isDepthPositive, linearizeOplus in core/dataTypes/optimization/OptimizableTypes.{hpp,cpp}); from
// g2o it needs only the containers those functions read and write: the edge's two vertex
// pointers, measurement, error, information and Jacobian members, the vertices' estimates, and
// SE3Quat's map() and rotation().  SE3Quat keeps a unit quaternion with w >= 0 and a translation,
// map(X) = q X + t, as g2o's does.  VertexSE3Expmap::oplusImpl restates g2o's published update
// T <- exp(delta) T (delta = [omega; upsilon], Rodrigues forms, R = V = I + W + W^2 below
// |omega| = 1e-5); it is defined so the vertex subclasses link, and the pin does not rely on it.
#pragma once

#include <cmath>
#include <iostream>
#include <vector>

#include <ref_eigen.hpp>

namespace g2o {

typedef Eigen::Matrix<double, 6, 1> Vector6d;

class SE3Quat {
public:
    SE3Quat() = default;
    SE3Quat(const Eigen::Matrix3d& R, const Eigen::Vector3d& t) : r_(Eigen::Quaterniond(R)), t_(t) {
        normalizeRotation();
    }
    SE3Quat(const Eigen::Quaterniond& q, const Eigen::Vector3d& t) : r_(q), t_(t) { normalizeRotation(); }

    const Eigen::Vector3d& translation() const { return t_; }
    const Eigen::Quaterniond& rotation() const { return r_; }
    void setTranslation(const Eigen::Vector3d& t) { t_ = t; }
    void setRotation(const Eigen::Quaterniond& q) {
        r_ = q;
        normalizeRotation();
    }

    Eigen::Vector3d map(const Eigen::Vector3d& xyz) const { return r_ * xyz + t_; }

    SE3Quat operator*(const SE3Quat& b) const {
        SE3Quat r;
        r.r_ = r_ * b.r_;
        r.t_ = t_ + r_ * b.t_;
        r.normalizeRotation();
        return r;
    }

    void normalizeRotation() {
        if (r_.w() < 0) r_ = Eigen::Quaterniond(-r_.w(), -r_.x(), -r_.y(), -r_.z());
        r_.normalize();
    }

    // exp of a twist [omega; upsilon] (rotation first).
    static SE3Quat exp(const Vector6d& update) {
        const Eigen::Vector3d omega(update[0], update[1], update[2]);
        const Eigen::Vector3d upsilon(update[3], update[4], update[5]);
        const double theta = omega.norm();
        Eigen::Matrix3d W;
        W << 0.0, -omega[2], omega[1], omega[2], 0.0, -omega[0], -omega[1], omega[0], 0.0;
        const Eigen::Matrix3d W2 = W * W;
        const Eigen::Matrix3d I = Eigen::Matrix3d::Identity();
        Eigen::Matrix3d R, V;
        if (theta < 1e-5) {
            R = I + W + W2;
            V = R;
        } else {
            const double t2 = theta * theta;
            R = I + W * (std::sin(theta) / theta) + W2 * ((1.0 - std::cos(theta)) / t2);
            V = I + W * ((1.0 - std::cos(theta)) / t2) + W2 * ((theta - std::sin(theta)) / (t2 * theta));
        }
        return SE3Quat(Eigen::Quaterniond(R), V * upsilon);
    }

private:
    Eigen::Quaterniond r_;
    Eigen::Vector3d t_;
};

struct HyperGraph {
    struct Vertex {
        virtual ~Vertex() = default;
        int id = -1;
    };
};

struct OptimizableGraph {
    struct Vertex : HyperGraph::Vertex {
        virtual void oplusImpl(const double* update) = 0;
        void setId(int i) { id = i; }
        void setFixed(bool f) { fixed_ = f; }
        void setMarginalized(bool m) { marginalized_ = m; }
        bool fixed() const { return fixed_; }

    private:
        bool fixed_ = false, marginalized_ = false;
    };
};

template <int D, class T>
class BaseVertex : public OptimizableGraph::Vertex {
public:
    static const int Dimension = D;
    typedef T EstimateType;
    const T& estimate() const { return _estimate; }
    void setEstimate(const T& e) { _estimate = e; }

protected:
    T _estimate;
};

class VertexSE3Expmap : public BaseVertex<6, SE3Quat> {
public:
    void oplusImpl(const double* update_) override {
        Vector6d u;
        for (int k = 0; k < 6; ++k) u[k] = update_[k];
        setEstimate(SE3Quat::exp(u) * estimate());
    }
};

class VertexSBAPointXYZ : public BaseVertex<3, Eigen::Vector3d> {
public:
    void oplusImpl(const double* update) override {
        for (int k = 0; k < 3; ++k) _estimate[k] += update[k];
    }
};

template <int D, class E>
class BaseEdge {
public:
    typedef E Measurement;
    typedef Eigen::Matrix<double, D, 1> ErrorVector;
    typedef Eigen::Matrix<double, D, D> InformationType;

    BaseEdge() : _information(InformationType::Identity()) {}
    virtual ~BaseEdge() = default;

    virtual void computeError() = 0;
    virtual void linearizeOplus() = 0;
    virtual bool read(std::istream& is) = 0;
    virtual bool write(std::ostream& os) const = 0;

    void setMeasurement(const Measurement& m) { _measurement = m; }
    const Measurement& measurement() const { return _measurement; }
    const ErrorVector& error() const { return _error; }
    InformationType& information() { return _information; }
    const InformationType& information() const { return _information; }
    void setInformation(const InformationType& i) { _information = i; }
    double chi2() const {
        double s = 0.0;
        for (int i = 0; i < D; ++i)
            for (int j = 0; j < D; ++j) s += _error[i] * _information(i, j) * _error[j];
        return s;
    }
    void setVertex(int k, HyperGraph::Vertex* v) { _vertices[k] = v; }

protected:
    std::vector<HyperGraph::Vertex*> _vertices;
    Measurement _measurement;
    ErrorVector _error;
    InformationType _information;
};

template <int D, class E, class VertexXi, class VertexXj>
class BaseBinaryEdge : public BaseEdge<D, E> {
public:
    typedef Eigen::Matrix<double, D, VertexXi::Dimension> JacobianXiOplusType;
    typedef Eigen::Matrix<double, D, VertexXj::Dimension> JacobianXjOplusType;

    BaseBinaryEdge() { this->_vertices.assign(2, nullptr); }

    const JacobianXiOplusType& jacobianOplusXi() const { return _jacobianOplusXi; }
    const JacobianXjOplusType& jacobianOplusXj() const { return _jacobianOplusXj; }

protected:
    JacobianXiOplusType _jacobianOplusXi;
    JacobianXjOplusType _jacobianOplusXj;
};

}  // namespace g2o
