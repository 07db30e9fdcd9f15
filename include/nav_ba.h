/*
 * nav_ba.h - C ABI of the GB300 bundle-adjustment back end.
 *
 * This library replaces the arithmetic that nav24's graph back end hands to g2o:
 *   NAV24::BE::GraphOptim::solve(const ProblemPtr&)      core/backEnd/BE_GraphOptim.cpp:31-77
 * for a PR_VBA problem (core/backEnd/Problem.hpp:107-113): keyframe poses, map points and the
 * observation graph go in, optimized poses and points come out.  Everything is plain C: host
 * pointers, sizes and integer status codes.  No exception crosses this boundary.
 *
 * Conventions
 *  - A pose is T_cw (world -> camera), passed as 12 doubles: the row-major 3x4 block [R | t]
 *    of nav24's 4x4 PoseSE3 (core/trajectory/pose/Pose.hpp:104, read at BE_GraphOptim.cpp:91-93).
 *  - Observations are undistorted pixel measurements (KeyPoint2D::getPointUd,
 *    core/sensorData/observation/Point2D.hpp:23) with the camera and point they link.
 *    Observation order is the edge order; any order is accepted.
 *  - The residual of one observation is e = z - pi(T_cw * X_w) (core/dataTypes/optimization/
 *    OptimizableTypes.hpp:102-107) with the pinhole projection of core/sensor/camera/models/
 *    Pinhole.cpp:30-36.  The information matrix is the identity (BE_GraphOptim.cpp:188-189).
 *  - The cost is g2o's robust chi2: sum over active edges of rho(e^T e), rho = identity or Huber.
 *  - All arithmetic at this boundary is FP64.  nav24 rounds points and measurements to float
 *    on the way in and points to float on the way out (BE_GraphOptim.cpp:147,239); that rounding
 *    belongs to the caller's adapter (nav24_gb300/adapter/GraphOptimGpu.cpp does it).
 *
 * Threading: one context per host thread.  A context owns one CUDA stream and its device
 * buffers; every call on it is synchronous (it returns after results are on the host).  Device
 * and page-locked buffers are kept across calls and grow to the largest call (a large-problem
 * solve's buffers included); nav_ba_destroy frees them.
 */
#ifndef NAV_BA_H
#define NAV_BA_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define NAV_BA_ABI_VERSION 2

typedef enum nav_ba_status {
    NAV_BA_OK = 0,
    /* No pose, or no point with an edge: nothing is optimized and the outputs are copies of
     * the inputs.  nav24 logs a warning and returns in this case (BE_GraphOptim.cpp:59-63). */
    NAV_BA_EMPTY = 1,
    NAV_BA_ERR_ARGUMENT = -1,          /* null pointer, negative size, index out of range      */
    NAV_BA_ERR_NONFINITE_INPUT = -2,   /* NaN/Inf in a pose, point, observation or intrinsic   */
    NAV_BA_ERR_NONFINITE_COST = -3,    /* the initial cost is not finite (e.g. a point at Z=0) */
    NAV_BA_ERR_CUDA = -4,              /* a CUDA runtime call failed                           */
    NAV_BA_ERR_OUT_OF_MEMORY = -5,     /* device or pinned-host allocation failed              */
    NAV_BA_ERR_UNSUPPORTED = -6,       /* size beyond an engine limit or option combination    */
    NAV_BA_ERR_DEVICE_TIMEOUT = -7,    /* a bounded device-side wait ran out                   */
    NAV_BA_ERR_NO_DEVICE = -8          /* no CUDA device, or the device index is invalid       */
} nav_ba_status;

/* Camera models.  PINHOLE is nav24's Pinhole (Pinhole.cpp:30-36,70-80).  PINHOLE_RADIAL adds
 * the two-coefficient radial factor d = 1 + k1 r^2 + k2 r^4 on normalized coordinates; it has
 * no counterpart in nav24's BA (nav24 undistorts before BA, Calibration.cpp:135-148).
 * KANNALA_BRANDT8 is nav24's fisheye model (core/sensor/camera/models/KannalaBrandt8.cpp:80-107,
 * Jacobian :195-226, selected at Calibration.cpp:81-82) with intrinsics fx, fy, cx, cy, k1..k4:
 * pi = f r(theta) (x, y)/rho + c, theta = atan2(rho, z), r = theta + k1 theta^3 + ... + k4 theta^9,
 * evaluated in the engine's precision (the reference rounds theta and psi to float). */
typedef enum nav_ba_camera_model {
    NAV_BA_CAM_PINHOLE = 0,
    NAV_BA_CAM_PINHOLE_RADIAL = 1,
    NAV_BA_CAM_KANNALA_BRANDT8 = 2
} nav_ba_camera_model;

typedef enum nav_ba_precision {
    NAV_BA_FP64 = 0,   /* plain: every kernel in FP64                                        */
    NAV_BA_MIXED = 1   /* FP32 residuals/Jacobians/Hessian blocks; FP64 reduced-system
                          Cholesky, cost, gain ratio and SE(3) update                         */
} nav_ba_precision;

typedef enum nav_ba_solver {
    NAV_BA_SOLVER_CHOLESKY = 0,  /* Schur complement + FP64 Cholesky of the reduced system
                                    (g2o BlockSolver_6_3 + LinearSolverEigen,
                                    BE_GraphOptim.cpp:41-45)                                  */
    NAV_BA_SOLVER_PCG = 1        /* matrix-free Schur + block-Jacobi preconditioned CG        */
} nav_ba_solver;

/* Why the Levenberg-Marquardt loop stopped (g2o OptimizationAlgorithmLevenberg::solve). */
typedef enum nav_ba_termination {
    NAV_BA_TERM_ITERATIONS = 0,        /* ran the requested number of iterations           */
    NAV_BA_TERM_TRIALS_EXHAUSTED = 1,  /* an iteration used all its damping trials          */
    NAV_BA_TERM_ZERO_GAIN = 2,         /* gain ratio exactly zero (no change in cost)       */
    NAV_BA_TERM_LAMBDA_NONFINITE = 3,  /* damping overflowed                                */
    NAV_BA_TERM_NOTHING_TO_DO = 4      /* no free vertex (all fixed) or an empty problem    */
} nav_ba_termination;

/* One BA problem (nav24: PR_VBA frames + calibration, Problem.hpp:107-113). */
typedef struct nav_ba_problem {
    int32_t n_cams;
    int32_t n_points;
    int32_t n_obs;
    const double* cam_pose;       /* [n_cams][12] row-major [R|t] of T_cw                   */
    const uint8_t* cam_fixed;     /* [n_cams] 1 = fixed (Frame::isOptFixed); NULL: none     */
    const double* points;         /* [n_points][3] world coordinates                        */
    const uint8_t* point_fixed;   /* [n_points] 1 = fixed; NULL: none                       */
    const double* obs_uv;         /* [n_obs][2] measured pixel (u, v)                       */
    const int32_t* obs_cam;       /* [n_obs] camera index of each observation               */
    const int32_t* obs_point;     /* [n_obs] point index of each observation                */
    int32_t camera_model;         /* nav_ba_camera_model                                    */
    int32_t reserved0;
    double intrinsics[8];         /* fx, fy, cx, cy, k1, k2, 0, 0 (KANNALA_BRANDT8: k1..k4)  */
} nav_ba_problem;

typedef struct nav_ba_options {
    int32_t iterations;           /* LM iterations (Problem::getNumIter, Problem.hpp:93)   */
    int32_t precision;            /* nav_ba_precision                                       */
    int32_t solver;               /* nav_ba_solver                                          */
    int32_t robust;               /* 1: Huber kernel on every edge (PR_VBA::mbRobust)       */
    double huber_delta;           /* Huber threshold in pixels (nav24: float(sqrt(5.99)))   */
    double initial_lambda;        /* > 0: first damping used as given; <= 0: tau*max diag   */
    double tau;                   /* g2o default 1e-5                                        */
    int32_t max_trials;           /* damping trials per iteration (g2o default 10)           */
    int32_t optimize_distortion;  /* 1: k1,k2 shared by all cameras are optimized            */
    double pcg_tolerance;         /* relative residual for NAV_BA_SOLVER_PCG                 */
    int32_t pcg_max_iterations;
    int32_t deterministic;        /* 1 (default): fixed-order reductions, bitwise repeatable */
    int32_t reserved[8];
} nav_ba_options;

typedef struct nav_ba_result {
    /* outputs, each may be NULL */
    double* cam_pose_out;         /* [n_cams][12] optimized T_cw (fixed cameras: unchanged)   */
    double* points_out;           /* [n_points][3] optimized points                          */
    double* intrinsics_out;       /* [8] (k1,k2 change only with optimize_distortion)         */
    double* cost_trace;           /* [iterations + 1]: cost before iteration 0, then after
                                     each iteration that ran                                 */
    /* statistics, always written */
    double initial_cost;
    double final_cost;
    double final_lambda;
    double time_setup_ms;         /* host-side structure build and upload (batches of >= 64
                                     windows: until the last part is launched, the device
                                     already solving the earlier parts)                     */
    double time_solve_ms;         /* device LM loop (pipelined batches: the waits for the
                                     parts' streams after setup)                            */
    double time_download_ms;      /* results to the caller (pipelined batches: each part
                                     read back while the later parts still run)             */
    int32_t iterations_done;
    int32_t trials_accepted;
    int32_t trials_rejected;
    int32_t termination;          /* nav_ba_termination                                     */
    int32_t n_active_edges;       /* edges in the cost (not both vertices fixed)            */
    int32_t n_free_cams;
    int32_t n_free_points;
    int32_t n_schur_blocks;       /* stored lower-triangle 6x6 blocks of the reduced system */
    int32_t pcg_iterations_total;
    int32_t status;               /* nav_ba_status of this problem (batched calls)          */
    int64_t edge_iterations;      /* active edges x LM iterations done (nav_ba_run: summed) */
    int64_t h2d_bytes;            /* bytes this call copied host -> device                  */
    int64_t d2h_bytes;            /* bytes this call copied device -> host                  */
    /* active edges whose point lies at or behind its camera (Z <= 0 in the camera frame) at the
     * final state: the edges for which EdgeSE3ProjectXYZ::isDepthPositive
     * (core/dataTypes/optimization/OptimizableTypes.hpp:109-113) is false.  nav24's GraphOptim never
     * calls that test; ORB-SLAM-style callers use it after a solve to drop such edges. */
    int32_t n_depth_nonpositive;
    int32_t reserved1;
} nav_ba_result;

typedef struct nav_ba_ctx nav_ba_ctx;

/* Fill *opt with the defaults of nav24's call: 5 iterations (Problem.hpp:84), FP64, Cholesky,
 * no robust kernel (PR_VBA::mbRobust = false), Huber delta float(sqrt(5.99)) (BE_GraphOptim.cpp:125),
 * tau-initialised damping, 10 trials. */
void nav_ba_options_default(nav_ba_options* opt);

/* Create a context on CUDA device `device`.  Replaces the per-call g2o optimizer construction
 * (BE_GraphOptim.cpp:40-49); one context may serve many solves. */
nav_ba_status nav_ba_create(nav_ba_ctx** ctx, int32_t device);
void nav_ba_destroy(nav_ba_ctx* ctx);

/* Solve one problem: replaces GraphOptim::solve's graph build (BE_GraphOptim.cpp:51-57),
 * optimizer.initializeOptimization/optimize(n) (:67-68) and the write-back (:73-76).
 * Synchronous.  On any error status the outputs are left untouched. */
nav_ba_status nav_ba_solve(nav_ba_ctx* ctx, const nav_ba_problem* problem,
                           const nav_ba_options* options, nav_ba_result* result);

/* Solve n_windows independent problems (sliding-window BA of FE_SlamMonoV.cpp:143-166, one
 * window per tracked frame) in one device launch sequence.  results[i] belongs to windows[i].
 * Each window is solved exactly as nav_ba_solve would solve it alone.  Windows up to
 * NAV_BA_WINDOW_MAX_CAMS free cameras use the batched window engine. */
#define NAV_BA_WINDOW_MAX_CAMS 24
nav_ba_status nav_ba_solve_batched(nav_ba_ctx* ctx, const nav_ba_problem* windows,
                                   int32_t n_windows, const nav_ba_options* options,
                                   nav_ba_result* results);

/* Two-phase form of nav_ba_solve for callers that solve the same graph repeatedly:
 * nav_ba_prepare builds the structure and uploads the initial state; nav_ba_run runs the
 * LM loop from that uploaded state on the device (no host transfer of the problem), and
 * nav_ba_fetch copies the last run's results to the host. */
nav_ba_status nav_ba_prepare(nav_ba_ctx* ctx, const nav_ba_problem* problem,
                             const nav_ba_options* options);
nav_ba_status nav_ba_run(nav_ba_ctx* ctx, const nav_ba_options* options, nav_ba_result* stats);
nav_ba_status nav_ba_fetch(nav_ba_ctx* ctx, nav_ba_result* result);

/* Batched form of nav_ba_prepare: windows as in nav_ba_solve_batched.  nav_ba_run then solves
 * all of them in one launch (stats of the whole batch: summed iterations/trials, summed costs,
 * the launch time); nav_ba_fetch_batched copies every window's results. */
nav_ba_status nav_ba_prepare_batched(nav_ba_ctx* ctx, const nav_ba_problem* windows,
                                     int32_t n_windows, const nav_ba_options* options);
nav_ba_status nav_ba_fetch_batched(nav_ba_ctx* ctx, nav_ba_result* results);

/* Residuals and Jacobians of every observation at the problem's initial state, computed by
 * the device linearization kernel in the given precision (EdgeSE3ProjectXYZ::computeError and
 * ::linearizeOplus, OptimizableTypes.hpp:102-107, OptimizableTypes.cpp:140-161).
 *   e  [n_obs][2], jc [n_obs][2][6] (pose, rotation first), jp [n_obs][2][3] (point),
 *   w  [n_obs] robust weight rho'(e^T e) (1 without a robust kernel).  Any may be NULL. */
nav_ba_status nav_ba_linearize(nav_ba_ctx* ctx, const nav_ba_problem* problem,
                               const nav_ba_options* options, double* e, double* jc,
                               double* jp, double* w);

/* Reduced camera system at the initial state for damping `lambda`, assembled on the device:
 * S = U + lambda I - W (V + lambda I)^-1 W^T and b' (g2o BlockSolver::solve's Schur step).
 * Free cameras are numbered in input order; s is [6 nf][6 nf] row-major (both triangles), b is
 * [6 nf], cam_index [n_cams] receives each camera's free index or -1.  *n_free receives nf;
 * s and b are written only when capacity_free >= nf. */
nav_ba_status nav_ba_reduced_system(nav_ba_ctx* ctx, const nav_ba_problem* problem,
                                    const nav_ba_options* options, double lambda,
                                    int32_t capacity_free, int32_t* n_free, double* s,
                                    double* b, int32_t* cam_index);

/* Robust chi2 of the problem's initial state, evaluated on the device in FP64. */
nav_ba_status nav_ba_cost(nav_ba_ctx* ctx, const nav_ba_problem* problem,
                          const nav_ba_options* options, double* cost);

/* No counterpart in the reference (nav24 builds a g2o optimizer on the heap for every call).
 * nav_ba_solve for callers that must not allocate device memory while solving: a tracking
 * thread with a real-time budget (cudaMalloc/cudaFree can block, cudaFree synchronizes the
 * device), or a process whose device memory is reserved by another framework's allocator.
 * It solves one window with the window engine, and every device buffer it uses lives in one
 * static device array of NAV_BA_NOALLOC_ARENA_BYTES that each GPU loading the library holds until
 * the process exits.  No cudaMalloc, cudaFree or other allocating routine is called.
 * Limits: NAV_BA_NOALLOC_MAX_CAMS cameras (at most NAV_BA_WINDOW_MAX_CAMS free),
 * NAV_BA_NOALLOC_MAX_POINTS points, NAV_BA_NOALLOC_MAX_OBS observations and
 * NAV_BA_NOALLOC_MAX_PAIRS Schur pairs, and the whole layout must fit the array; larger problems
 * are rejected with NAV_BA_ERR_UNSUPPORTED and a message.  Cholesky solver only, no distortion
 * optimization.  The first call on a device looks up the array's device address (make that first
 * call before any stream capture).  All calls on a device share the array; calls whose GPU work
 * overlaps (e.g. from two contexts on one device) race on it. */
#define NAV_BA_NOALLOC_MAX_CAMS 64
#define NAV_BA_NOALLOC_MAX_POINTS 4096
#define NAV_BA_NOALLOC_MAX_OBS 32768
#define NAV_BA_NOALLOC_MAX_PAIRS 262144
#define NAV_BA_NOALLOC_ARENA_BYTES (16u * 1024u * 1024u)
nav_ba_status nav_ba_solve_noalloc(nav_ba_ctx* ctx, const nav_ba_problem* problem,
                                   const nav_ba_options* options, nav_ba_result* result);

/* ---- motion-only BA (per-frame tracking) ------------------------------------------------------
 *
 * One free pose against fixed world points: nav24's EdgeSE3ProjectXYZOnlyPose (declared, commented
 * out, in core/dataTypes/optimization/OptimizableTypes.hpp:34-60; linearizeOplus at
 * OptimizableTypes.cpp:50-64: e = z - pi(T Xw), J = -Jpi [-[Xc]x | I]), the problem of the tracking call
 * core/frontEnd/FE_SlamMonoV.cpp:153-165 when the current frame is optimized against a fixed map.
 * The LM is the one of nav_ba_solve (iterations, robust kernel, damping, trials, precision), on the
 * 6x6 normal equations.  nav_ba_solve_pose_batched solves n problems in one launch (one block each).
 * Statuses per problem as in nav_ba_solve_batched; a problem with no observation is EMPTY. */
typedef struct nav_ba_pose_problem {
    int32_t n_obs;
    int32_t camera_model;         /* NAV_BA_CAM_PINHOLE or NAV_BA_CAM_PINHOLE_RADIAL (k1, k2 fixed) */
    const double* pose;           /* [12] initial T_cw                                          */
    const double* points;         /* [n_obs][3] fixed world point of each observation          */
    const double* obs_uv;         /* [n_obs][2]                                                 */
    double intrinsics[8];         /* fx, fy, cx, cy, k1, k2, 0, 0                               */
} nav_ba_pose_problem;

typedef struct nav_ba_pose_result {
    double* pose_out;             /* [12] optimized T_cw, or NULL                              */
    double initial_cost;
    double final_cost;
    double final_lambda;
    int32_t iterations_done;
    int32_t trials_accepted;
    int32_t trials_rejected;
    int32_t termination;          /* nav_ba_termination                                         */
    int32_t status;               /* nav_ba_status of this problem                              */
    int32_t n_depth_nonpositive;  /* observations behind the final pose (Z <= 0), as nav_ba_result */
} nav_ba_pose_result;

nav_ba_status nav_ba_solve_pose_batched(nav_ba_ctx* ctx, const nav_ba_pose_problem* problems,
                                        int32_t n_problems, const nav_ba_options* options,
                                        nav_ba_pose_result* results);

/* ---- two-view triangulation and hypothesis check (map initialization) --------------------------
 *
 * The per-match work of TwoViewReconstruction::CheckRT (core/operators/mapInit/
 * OP_2ViewReconstruction.cpp:1244-1353) with Triangulate (:1179-1193), for n_hyp relative-pose
 * hypotheses (R, t of camera 2 with respect to camera 1, e.g. the 4 of ReconstructF or the 8 of
 * ReconstructH) and n_matches matches at once.  Per hypothesis and match: the DLT point of
 * A = [x1 P1_3 - P1_1; y1 P1_3 - P1_2; x2 P2_3 - P2_1; y2 P2_3 - P2_2] (P1 = K[I|0], P2 = K[R|t]) as the
 * right singular vector of A's smallest singular value (one-sided Jacobi SVD, FP64), then the checks
 * in CheckRT's order:
 * finite, depth > 0 in camera 1 and camera 2 unless the parallax is below the minimum, squared
 * reprojection error <= th2 in both images.  A match that passes is "triangulated" (counted in
 * n_good); it is also "good" (vbGood) when cos(parallax) < min_parallax_cos.  parallax_deg is
 * CheckRT's statistic: acos of the sorted cos-parallax values at index min(min_triangulated, n - 1),
 * in degrees (0 when no match passes). */
typedef struct nav_ba_twoview {
    int32_t n_matches;
    int32_t n_hyp;
    double K[4];                  /* fx, fy, cx, cy                                             */
    const double* kp1;            /* [n_matches][2] pixel in image 1                            */
    const double* kp2;            /* [n_matches][2] pixel in image 2                            */
    const uint8_t* inlier;        /* [n_matches] vbMatchesInliers, or NULL (all)                */
    const double* R;              /* [n_hyp][9] row-major                                       */
    const double* t;              /* [n_hyp][3]                                                 */
    double th2;                   /* squared reprojection threshold (CheckRT: 4 sigma^2)        */
    double min_parallax_cos;      /* mMinParallaxCRT                                            */
    int32_t min_triangulated;     /* mMinTriangulated                                           */
    int32_t reserved;
} nav_ba_twoview;

typedef struct nav_ba_twoview_result {
    double* points;               /* [n_hyp][n_matches][3] point in camera 1 (of every match
                                     whose DLT point is finite; NaN otherwise), or NULL         */
    uint8_t* triangulated;        /* [n_hyp][n_matches] passed every check, or NULL            */
    uint8_t* good;                /* [n_hyp][n_matches] vbGood, or NULL                        */
    int32_t* n_good;              /* [n_hyp] nGood                                              */
    double* parallax_deg;         /* [n_hyp]                                                    */
} nav_ba_twoview_result;

nav_ba_status nav_ba_twoview_check(nav_ba_ctx* ctx, const nav_ba_twoview* in, nav_ba_twoview_result* out);

/* ---- keypoint undistortion (the measurements BA consumes) ------------------------------------
 *
 * Calibration::undistort (core/sensor/camera/Calibration.cpp:135-148) -> PinholeRadTan::
 * UndistortKeyPoints (core/sensor/camera/models/PinholeRadTan.cpp:11-24) -> cv::undistortPoints
 * with R = I and P = K: the fixed-point inversion of the radial-tangential model on normalized
 * coordinates, x <- (x_d - dx(x)) / (1 + k1 r^2 + k2 r^4), `iterations` times (OpenCV's default: 5),
 * mapped back through K; FP64.  K = fx, fy, cx, cy; dist = k1, k2, p1, p2 (the 4-coefficient order
 * of mD_cv).  uv_in and uv_out are [n][2] and may be the same array. */
nav_ba_status nav_ba_undistort_points(nav_ba_ctx* ctx, const double* K, const double* dist,
                                      int32_t iterations, int32_t n, const double* uv_in,
                                      double* uv_out);

/* ---- differentiation through the LM steps (no counterpart in the reference) ----------------
 *
 * The differentiable function is the LM solve with its damping schedule frozen: the steps that
 * the solve accepted, each x <- x [+] dx with (H(x) + lambda I) dx = b(x) at its recorded lambda.
 * Rejected trials leave the state unchanged and so are not part of the function.  Outputs are the
 * final robust cost, the poses and the points; inputs whose gradients are given are the
 * observations, the intrinsics (fx, fy, cx, cy) and the initial poses and points.
 *
 * nav_ba_vjp runs the forward and, when `cot` and `grads` are both non-NULL, the backward:
 *   - schedule->replay == 0: the forward is the LM solve of nav_ba_solve (same semantics, run by
 *     the whole-GPU engine, so it agrees with nav_ba_solve to rounding) and schedule receives the
 *     damping of each accepted step;
 *   - schedule->replay == 1: the forward applies the schedule's n_steps steps unconditionally
 *     (result->iterations_done = n_steps).  Replaying a recorded schedule on the same inputs
 *     reproduces the recorded solve, and is the function that finite differences check.
 * The backward is the adjoint of the unrolled steps: per step (last first) it re-linearizes at
 * the stored state (Jacobians are recomputed, not stored), refactors H + lambda I, solves the
 * adjoint system with that factorization, and accumulates per-observation adjoints of the
 * residual, Jacobian and Huber weight.  L = cot->cost * final_cost + <cot->cam_pose, cam_pose_out>
 * + <cot->points, points_out>.
 * Supported: FP64 precision, the Cholesky solver, the pinhole model, no distortion optimization;
 * other options return NAV_BA_ERR_UNSUPPORTED.  An EMPTY problem writes the inputs as outputs and
 * zero gradients. */
#define NAV_BA_VJP_MAX_STEPS 64
typedef struct nav_ba_schedule {
    int32_t replay;                        /* 0: run LM and record; 1: apply the given steps   */
    int32_t n_steps;                       /* accepted steps (<= NAV_BA_VJP_MAX_STEPS)          */
    double lambda[NAV_BA_VJP_MAX_STEPS];   /* damping of each accepted step                     */
} nav_ba_schedule;

typedef struct nav_ba_cotangent {
    double cost;                  /* dL / d final cost                                         */
    const double* cam_pose;       /* [n_cams][12] dL / d cam_pose_out entries, or NULL (zero)  */
    const double* points;         /* [n_points][3] dL / d points_out, or NULL (zero)           */
} nav_ba_cotangent;

typedef struct nav_ba_grads {
    double* obs_uv;               /* [n_obs][2] dL / d obs_uv, or NULL                         */
    double intrinsics[8];         /* dL / d (fx, fy, cx, cy); entries 4..7 are 0               */
    /* The next two are gradients with respect to the initial values of the optimized vertices
     * (cameras and points that are free and have an active edge); 0 for the other vertices. */
    double* cam_tangent;          /* [n_cams][6] dL / d (left perturbation [omega; upsilon] of
                                     each input pose: T -> exp(eps) T), or NULL                  */
    double* points;               /* [n_points][3] dL / d input points, or NULL                */
} nav_ba_grads;

nav_ba_status nav_ba_vjp(nav_ba_ctx* ctx, const nav_ba_problem* problem,
                         const nav_ba_options* options, nav_ba_schedule* schedule,
                         const nav_ba_cotangent* cot, nav_ba_result* result, nav_ba_grads* grads);

/* Last error message of the context (empty string if none). */
const char* nav_ba_last_error(const nav_ba_ctx* ctx);
const char* nav_ba_status_string(nav_ba_status status);
int32_t nav_ba_abi_version(void);

#ifdef __cplusplus
}
#endif

#endif /* NAV_BA_H */
