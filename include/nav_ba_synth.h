/*
 * nav_ba_synth.h - seeded synthetic bundle-adjustment problems.
 *
 * nav24 ships no BA dataset and no BA test (its examples drive BA from live ORB tracking,
 * core/frontEnd/FE_SlamMonoV.cpp:143-166 and core/operators/mapInit/OP_MapInitialization.cpp:
 * 196-204), so every workload here is synthetic.  Five geometry families:
 *   0  ring     : cameras on a circle looking at the origin, points in a cube      (global BA)
 *   1  grid     : downward cameras on a grid over a ground patch                   (large window)
 *   2  windows  : many independent short trajectories, points in a box ahead       (local BA)
 *   3  cap      : cameras on a sphere cap looking at the centre                    (differentiable)
 *   4  eight    : a three-loop figure-eight with radial distortion and outliers    (large robust)
 * A problem is a plain struct-of-arrays; batched problems (family 2) are windows laid out one
 * after another, with per-window offsets and window-local camera/point indices.
 */
#ifndef NAV_BA_SYNTH_H
#define NAV_BA_SYNTH_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct nav_synth_params {
    int32_t family;          /* 0..4 */
    int32_t n_cams;          /* 0: family default (family 2: maximum keyframes per window)  */
    int32_t n_points;        /* 0: family default (family 2: maximum points per window)     */
    int32_t n_windows;       /* family 2 only; 0: default 512                                */
    uint64_t seed;
    double pixel_noise;      /* < 0: family default (sigma in pixels)                        */
    double outlier_frac;     /* < 0: family default                                          */
    double rot_perturb;      /* < 0: default 0.01 rad (axis-angle sigma per axis)            */
    double trans_perturb;    /* < 0: default 0.05 m                                          */
    double point_perturb;    /* < 0: default 0.05 m                                          */
    int32_t min_cams;        /* family 2: minimum keyframes per window (0: 5)                 */
    int32_t min_points;      /* family 2: minimum points per window (0: 200)                  */
} nav_synth_params;

typedef struct nav_synth nav_synth;

/* Array identifiers for nav_synth_size / nav_synth_copy. */
enum {
    NAV_SYNTH_CAM_POSE = 0,       /* double [n_cams][12] initial (perturbed) T_cw           */
    NAV_SYNTH_CAM_POSE_TRUE = 1,  /* double [n_cams][12]                                    */
    NAV_SYNTH_CAM_FIXED = 2,      /* uint8  [n_cams]                                        */
    NAV_SYNTH_POINTS = 3,         /* double [n_points][3] initial                           */
    NAV_SYNTH_POINTS_TRUE = 4,    /* double [n_points][3]                                   */
    NAV_SYNTH_POINT_FIXED = 5,    /* uint8  [n_points]                                      */
    NAV_SYNTH_OBS_UV = 6,         /* double [n_obs][2]                                      */
    NAV_SYNTH_OBS_CAM = 7,        /* int32  [n_obs] (window-local index)                    */
    NAV_SYNTH_OBS_POINT = 8,      /* int32  [n_obs] (window-local index)                    */
    NAV_SYNTH_WIN_CAM_OFF = 9,    /* int64  [n_windows + 1]                                 */
    NAV_SYNTH_WIN_POINT_OFF = 10, /* int64  [n_windows + 1]                                 */
    NAV_SYNTH_WIN_OBS_OFF = 11,   /* int64  [n_windows + 1]                                 */
    NAV_SYNTH_INTRINSICS = 12,    /* double [8] true fx, fy, cx, cy, k1, k2, 0, 0           */
    NAV_SYNTH_INTRINSICS_INIT = 13, /* double [8] initial intrinsics (k1,k2 perturbed)      */
    NAV_SYNTH_N_ARRAYS = 14
};

/* Generate; returns NULL on invalid parameters.  Deterministic for a given seed. */
nav_synth* nav_synth_create(const nav_synth_params* params);
void nav_synth_destroy(nav_synth* s);
/* Scalars: n_windows, n_cams, n_points, n_obs (totals over windows), camera model. */
void nav_synth_counts(const nav_synth* s, int64_t* n_windows, int64_t* n_cams,
                      int64_t* n_points, int64_t* n_obs, int32_t* camera_model);
/* Element count of an array (elements, not bytes). */
int64_t nav_synth_size(const nav_synth* s, int32_t array_id);
/* Copy an array into dst (dst must hold nav_synth_size elements of the array's type). */
int32_t nav_synth_copy(const nav_synth* s, int32_t array_id, void* dst);

#ifdef __cplusplus
}
#endif

#endif /* NAV_BA_SYNTH_H */
