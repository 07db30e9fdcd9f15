// Stand-in for core/scene/worldObject/WorldObject.hpp:21-33.
#pragma once
#include <memory>
#include <vector>
#include "SmartObject.hpp"
#include "Observation.hpp"
namespace NAV24::WO {
class WorldObject : public SmartObject {
public:
    void addObservation(const OB::ObsPtr& p) { mvpObs.push_back(p); }
    std::vector<OB::ObsPtrW> getObservations() { return mvpObs; }
protected:
    std::vector<OB::ObsPtrW> mvpObs;
};
}  // namespace NAV24::WO
