// Stand-in for core/dataTypes/frame/Frame.hpp:16-42.
#pragma once
#include <memory>
#include <vector>
#include "Pose.hpp"
#include "Point2D.hpp"
namespace NAV24 {
class Frame : public SmartObject {
public:
    Frame() = default;
    Frame(double ts_, PosePtr pose, const std::vector<OB::ObsPtr>& vObs) : mvpObservations(vObs), mpPose(std::move(pose)), ts(ts_) {}
    [[nodiscard]] const std::vector<OB::ObsPtr>& getObservations() const { return mvpObservations; }
    virtual void setObservations(const std::vector<OB::ObsPtr>& v) { mvpObservations = v; }
    [[nodiscard]] const PosePtr& getPose() const { return mpPose; }
    void setPose(const PosePtr& p) { mpPose = p; }
    [[nodiscard]] double getTs() const { return ts; }
    [[nodiscard]] unsigned long getOptId() const { return mOptId; }
    void setOptId(const unsigned long& id) { mOptId = id; }
protected:
    std::vector<OB::ObsPtr> mvpObservations;
    PosePtr mpPose;
    double ts = -1.0;
    unsigned long mOptId = 0;
};
typedef std::shared_ptr<Frame> FramePtr;
}  // namespace NAV24
