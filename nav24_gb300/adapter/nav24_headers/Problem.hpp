// Stand-in for core/backEnd/Problem.hpp:16-47 (Problem, PR_VBA).
#pragma once
#include <memory>
#include <vector>
#include "Frame.hpp"
#include "Calibration.hpp"
namespace NAV24 {
class Problem {
public:
    virtual ~Problem() = default;
    [[nodiscard]] virtual bool isSolved() const { return solved; }
    virtual void setSolved(const bool s) { solved = s; }
    [[nodiscard]] int getNumIter() const { return nIterations; }
    void setNumIter(const int n) { nIterations = n; }
protected:
    bool solved = false;
    int nIterations = 5;
};
typedef std::shared_ptr<Problem> ProblemPtr;
class PR_VBA : public Problem {
public:
    PR_VBA(const std::vector<FramePtr>& vpFrames, const CalibPtr& pCalib) : mvpFrames(vpFrames), mpCalib(pCalib) {}
    std::vector<FramePtr> mvpFrames;
    CalibPtr mpCalib;
    bool mbRobust = false;
};
}  // namespace NAV24
