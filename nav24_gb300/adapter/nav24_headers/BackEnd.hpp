// Stand-in for core/backEnd/BackEnd.hpp:13-25 (the solve interface; the message hooks of
// MsgCallback are not needed by the adapter).
#pragma once
#include "Problem.hpp"
namespace NAV24::BE {
class BackEnd {
public:
    virtual ~BackEnd() = default;
    virtual void solve(const ProblemPtr& problem) = 0;
};
}  // namespace NAV24::BE
