// Stand-in for core/sensorData/observation/Observation.hpp:13-52.
#pragma once
#include <memory>
#include "SmartObject.hpp"
namespace NAV24 {
class Frame;
typedef std::shared_ptr<Frame> FramePtr;
typedef std::weak_ptr<Frame> FramePtrW;
}  // namespace NAV24
namespace NAV24::WO {
class WorldObject;
typedef std::shared_ptr<WorldObject> WoPtr;
typedef std::weak_ptr<WorldObject> WoPtrW;
}  // namespace NAV24::WO
namespace NAV24::OB {
class Observation : public SmartObject {
public:
    void setWorldObject(const WO::WoPtr& p) { mpWo = p; }
    WO::WoPtr getWorldObject() { return mpWo.lock(); }
    FramePtr getFrame() { return mpFrame.lock(); }
    void setFrame(const FramePtr& f) { mpFrame = f; }
protected:
    WO::WoPtrW mpWo;
    FramePtrW mpFrame;
};
typedef std::shared_ptr<Observation> ObsPtr;
typedef std::weak_ptr<Observation> ObsPtrW;
}  // namespace NAV24::OB
