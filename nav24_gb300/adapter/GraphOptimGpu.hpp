// GraphOptimGpu.hpp - drop-in replacement of nav24's graph back end (BE::GraphOptim,
// core/backEnd/BE_GraphOptim.hpp:19-34) that solves on the GPU through libnavba (include/nav_ba.h).
//
// Swap `std::make_shared<BE::GraphOptim>()` for `std::make_shared<BE::GraphOptimGpu>()` at the
// call sites (core/operators/mapInit/OP_MapInitialization.cpp:203-204,
// core/frontEnd/FE_SlamMonoV.cpp:164-165).  solve() takes the same PR_VBA problem and mutates the
// same objects: every posed frame gets a new PoseSE3 and optId -1, every point with an edge gets its
// float-rounded optimized position.
#pragma once

#include <memory>
#include <vector>

#include "BackEnd.hpp"
#include "Problem.hpp"
#include "nav_ba.h"

namespace NAV24::BE {

class GraphOptimGpu : public BackEnd {
public:
    // device: CUDA device index; precision: NAV_BA_FP64 (plain) or NAV_BA_MIXED.
    explicit GraphOptimGpu(int device = 0, int precision = NAV_BA_FP64);
    ~GraphOptimGpu() override;
    GraphOptimGpu(const GraphOptimGpu&) = delete;
    GraphOptimGpu& operator=(const GraphOptimGpu&) = delete;

    // BE::GraphOptim::solve (core/backEnd/BE_GraphOptim.cpp:31-77).
    void solve(const ProblemPtr& problem) override;

    // Several PR_VBA windows in one device launch.  The windows must not share frames or points
    // (each is written back as if solved alone).
    void solveBatched(const std::vector<ProblemPtr>& problems);

    // Status and statistics of the last solve (of each window for solveBatched).
    [[nodiscard]] nav_ba_status lastStatus() const { return mStatus; }
    [[nodiscard]] const std::vector<nav_ba_result>& lastResults() const { return mResults; }
    [[nodiscard]] const char* lastError() const;

    nav_ba_options options;  // iterations and robust kernel are taken from each problem

private:
    struct Flat;
    bool flatten(const ProblemPtr& problem, Flat& f);
    void recover(Flat& f, const nav_ba_result& r);

    nav_ba_ctx* mCtx = nullptr;
    nav_ba_status mStatus = NAV_BA_OK;
    std::vector<nav_ba_result> mResults;
};

}  // namespace NAV24::BE
