// structure.hpp - host-side graph build of a BA problem (the part of nav24's
// GraphOptim::solve that assembles the g2o graph, core/backEnd/BE_GraphOptim.cpp:79-211).
//
// From a nav_ba_problem it derives what the device engines consume:
//  * active edges: every observation, except those whose camera and point are both fixed
//    (g2o's initializeOptimization drops edges whose vertices are all fixed);
//  * free cameras: not fixed and with at least one active edge (numbered in input order);
//  * free points:  not fixed and with at least one active edge;
//  * the active edges grouped by point (point-major), input order within a point, with the
//    per-point edge ranges;
//  * the initial camera states (quaternion + translation + rotation) and points.
#pragma once

#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/nav_ba.h"
#include "ba_math.cuh"

namespace navba {

// One problem (window) laid out for the device.  All indices are window-local.
struct HostWindow {
    int32_t ncam = 0, npt = 0, ne = 0;
    int32_t nfc = 0, nfp = 0;
    std::vector<CamState> cam;        // [ncam]
    std::vector<int32_t> cam_free;    // [ncam] free index or -1
    std::vector<double> pt;           // [npt * 4] x y z 0
    std::vector<int32_t> pt_free;     // [npt] free index or -1
    std::vector<int32_t> pt_eoff;     // [npt + 1] edge range of each point (local)
    std::vector<int32_t> edge_cam;    // [ne] camera of each active edge
    std::vector<int32_t> edge_obs;    // [ne] observation index of each active edge
    std::vector<double> edge_uv;      // [ne * 2]
    std::vector<int32_t> edge_pt;     // [ne] point of each active edge
    int32_t n_schur_blocks = 0;       // lower-triangle co-visible free-camera block pairs
    int64_t n_pairs = 0;              // Schur pairs (i, j): same free point, free cameras,
                                      // free index of j's camera <= that of i's camera
};

// Validate a problem exactly like the oracle: pointers, sizes, index ranges, finiteness.
nav_ba_status validate_problem(const nav_ba_problem* p, std::string* why);
nav_ba_status validate_options(const nav_ba_options* o, std::string* why);

// Build the device layout of one problem (assumes validate_problem passed).
void build_window(const nav_ba_problem& p, const nav_ba_options& o, HostWindow& w);

}  // namespace navba
