// Stand-in for core/trajectory/pose/Pose.hpp:24-106 (Transformation, PoseSE3).
#pragma once
#include <memory>
#include <string>
#include <eigen3/Eigen/Dense>
namespace NAV24 {
namespace TF {
class Transformation {
public:
    Transformation(std::string ref_, std::string target_, double ts_) : ref(std::move(ref_)), target(std::move(target_)), ts(ts_) {}
    virtual ~Transformation() = default;
    [[nodiscard]] std::string getRef() const { return ref; }
    [[nodiscard]] std::string getTarget() const { return target; }
    [[nodiscard]] double getTimestamp() const { return ts; }
protected:
    std::string ref, target;
    double ts;
};
class PoseSE3 : public Transformation {
public:
    PoseSE3(const std::string& ref_, const std::string& target_, double ts_, Eigen::Matrix4d T_rt_)
        : Transformation(ref_, target_, ts_), T_rt(T_rt_) {}
    [[nodiscard]] Eigen::Matrix4d getPose() const { return T_rt; }
protected:
    Eigen::Matrix4d T_rt;
};
}  // namespace TF
typedef std::shared_ptr<TF::PoseSE3> PosePtr;
}  // namespace NAV24
