/*
 * ba_oracle.h - CPU FP64 oracle of nav24's bundle-adjustment back end.  TEST INFRASTRUCTURE:
 * only the tests, the smoke check and the CPU-baseline leg of bench.py may load it; the
 * product library never links it.
 *
 * The entry points take the same nav_ba_problem / nav_ba_options / nav_ba_result structs as
 * the product C ABI (include/nav_ba.h) so that every product call has an oracle twin.
 */
#ifndef NAV_BA_ORACLE_H
#define NAV_BA_ORACLE_H

#include "../include/nav_ba.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Full LM solve (the twin of nav_ba_solve).  n_threads >= 1 threads share the linearization,
 * the Schur complement and the cost; the factorization runs on one thread. */
int32_t oracle_solve(const nav_ba_problem* p, const nav_ba_options* o, nav_ba_result* r,
                     int32_t n_threads);

/* oracle_solve with a damping schedule (the twin of nav_ba_vjp's forward): sched->replay == 0
 * records the damping of every accepted step; sched->replay == 1 applies the given steps
 * unconditionally (x <- x [+] (H + lambda I)^-1 b at the current state, for each lambda). */
int32_t oracle_solve_schedule(const nav_ba_problem* p, const nav_ba_options* o, nav_ba_result* r,
                              int32_t n_threads, nav_ba_schedule* sched);

/* Twin of nav_ba_linearize (FP64). */
int32_t oracle_linearize(const nav_ba_problem* p, const nav_ba_options* o, double* e,
                         double* jc, double* jp, double* w);

/* oracle_linearize with a rounding mode: 0 = FP64 throughout (as oracle_linearize); 1 = the
 * reference's own roundings in KannalaBrandt8::project / projectJac (theta and psi through
 * atan2f/sqrtf, 3 k1 ... 9 k4 in float), to compare with nav24's code built in oracle/_ref. */
int32_t oracle_linearize_mode(const nav_ba_problem* p, const nav_ba_options* o, int32_t mode,
                              double* e, double* jc, double* jp, double* w);

/* Distortion-parameter Jacobian [n_obs][2][2] (d e / d (k1, k2)); radial model only. */
int32_t oracle_distortion_jacobian(const nav_ba_problem* p, double* jk);

/* Twin of nav_ba_reduced_system. */
int32_t oracle_reduced_system(const nav_ba_problem* p, const nav_ba_options* o, double lambda,
                              int32_t capacity_free, int32_t* n_free, double* s, double* b,
                              int32_t* cam_index);

/* Twin of nav_ba_cost. */
int32_t oracle_cost(const nav_ba_problem* p, const nav_ba_options* o, double* cost);

/* SE(3) helpers exposed for the tests: exp map update T <- exp(delta) * T in g2o's SE3Quat
 * semantics, on a 3x4 pose; and the pose -> quaternion -> pose round trip. */
void oracle_se3_update(const double* pose12, const double* delta6, double* out12);
void oracle_pose_roundtrip(const double* pose12, double* out12);

#ifdef __cplusplus
}
#endif

#endif
