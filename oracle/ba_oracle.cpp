// ba_oracle.cpp - CPU FP64 oracle of nav24's bundle-adjustment back end.
//
// TEST INFRASTRUCTURE.  Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load
// this library; the product (nav24_gb300/csrc) never links or calls it.
//
// Parity status: PINNED for the residual, the Jacobians and the SE(3) update against
// independently derived known answers (sympy differentiation of exp(delta)*T applied to a point,
// central finite differences) and against scipy's least_squares optimum; the LM schedule below
// restates g2o's published algorithm and is NOT pinned against g2o itself, which is absent from the
// reference tree (thirdparty/g2o is referenced by CMakeLists.txt:28 and core/CMakeLists.txt:102
// but not vendored, no version pinned) and cannot be built here.
//
// What this file restates, and from where:
//  * graph assembly (BE_GraphOptim.cpp:79-211): one pose vertex per camera, fixed flag from the
//    frame (:95); one point vertex per point with at least one edge (:204-209), fixed points are
//    fixed and not marginalized (:150-153); one edge per observation, Omega = I (:188-189),
//    optional Huber kernel (:191-195).
//  * residual e = z - pi(T.map(X)) (OptimizableTypes.hpp:102-107) with the pinhole projection
//    (Pinhole.cpp:30-36) and its Jacobian (Pinhole.cpp:70-80); edge Jacobians
//    (OptimizableTypes.cpp:140-161): J_point = -Jpi * R, J_pose = -Jpi * [ -[Xc]x | I ].
//  * g2o behaviour the reference relies on (ORB-SLAM2/3-bundled g2o fork; assumptions, stated
//    from g2o's published source and documentation):
//      - active edges exclude edges whose vertices are all fixed; vertices without an active
//        edge are not optimized (SparseOptimizer::initializeOptimization);
//      - robust chi2 = sum rho(e^T e); Huber rho(s) = s (s <= d^2), 2 d sqrt(s) - d^2 otherwise;
//        H and b are weighted by rho'(s) only (first order, BaseBinaryEdge::constructQuadraticForm);
//      - b = -J^T W e and the step solves (H + lambda I) dx = b (BlockSolver::setLambda adds
//        lambda to every diagonal entry, poses and points alike, before the Schur complement);
//      - Schur: S = Hpp - Hpl Hll^-1 Hlp, b' = bp - Hpl Hll^-1 bl, dx_l = Hll^-1 (bl - Hlp dx_p),
//        Hll^-1 of each 3x3 block by its adjugate (Eigen's fixed-size inverse);
//      - LM (OptimizationAlgorithmLevenberg::solve, Nielsen's rule as in Madsen, Nielsen &
//        Tingleff 2004): lambda0 = user value if > 0 else tau * max|diag H| (tau = 1e-5) on the
//        first iteration; up to maxTrialsAfterFailure = 10 trials; rho = (chi - chi_new) /
//        (dx^T (lambda dx + b) + 1e-3); accept if rho > 0 and chi_new finite:
//        lambda *= max(1/3, min(2/3, 1 - (2 rho - 1)^3)), nu = 2; else lambda *= nu, nu *= 2 and
//        restore; the trial loop runs while rho < 0; the outer loop stops when the trial count
//        reached the maximum, rho == 0, or lambda is not finite;
//      - VertexSE3Expmap::oplusImpl: T <- exp(delta) * T, delta = [omega; upsilon]; SE3Quat::exp
//        uses R = V = I + W + W^2 when |omega| < 1e-5 (g2o's small-angle branch) and the
//        Rodrigues forms otherwise; rotations are unit quaternions with w >= 0;
//        VertexSBAPointXYZ::oplusImpl: X += delta.
//  * the reduced camera system is factored by Cholesky (LL^T) inside its row envelope; the
//    reference's LinearSolverEigen (BE_GraphOptim.cpp:43) is a sparse LDL^T, which gives the same
//    solution up to rounding.
#include "ba_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#include <thread>
#include <vector>

namespace {

struct Quat {
    double x, y, z, w;
};
struct SE3 {
    Quat q;
    double t[3];
};

void normalize_rotation(Quat& q) {  // g2o SE3Quat::normalizeRotation
    if (q.w < 0) {
        q.x = -q.x; q.y = -q.y; q.z = -q.z; q.w = -q.w;
    }
    const double n = std::sqrt(q.x * q.x + q.y * q.y + q.z * q.z + q.w * q.w);
    q.x /= n; q.y /= n; q.z /= n; q.w /= n;
}

// Quaternion of a rotation matrix by Shepperd's method (J. Guidance & Control 1978): use the
// trace when positive, else the largest diagonal entry.  R row-major.
Quat quat_from_matrix(const double* R) {
    Quat q;
    const double tr = R[0] + R[4] + R[8];
    if (tr > 0.0) {
        double s = std::sqrt(tr + 1.0);
        q.w = 0.5 * s;
        s = 0.5 / s;
        q.x = (R[7] - R[5]) * s;
        q.y = (R[2] - R[6]) * s;
        q.z = (R[3] - R[1]) * s;
    } else {
        int i = 0;
        if (R[4] > R[0]) i = 1;
        if (R[8] > R[i * 4]) i = 2;
        const int j = (i + 1) % 3, k = (j + 1) % 3;
        double v[3];
        double s = std::sqrt(R[i * 4] - R[j * 4] - R[k * 4] + 1.0);
        v[i] = 0.5 * s;
        s = 0.5 / s;
        q.w = (R[k * 3 + j] - R[j * 3 + k]) * s;
        v[j] = (R[j * 3 + i] + R[i * 3 + j]) * s;
        v[k] = (R[k * 3 + i] + R[i * 3 + k]) * s;
        q.x = v[0]; q.y = v[1]; q.z = v[2];
    }
    return q;
}

void matrix_from_quat(const Quat& q, double* R) {
    const double tx = 2 * q.x, ty = 2 * q.y, tz = 2 * q.z;
    const double twx = tx * q.w, twy = ty * q.w, twz = tz * q.w;
    const double txx = tx * q.x, txy = ty * q.x, txz = tz * q.x;
    const double tyy = ty * q.y, tyz = tz * q.y, tzz = tz * q.z;
    R[0] = 1 - (tyy + tzz); R[1] = txy - twz;       R[2] = txz + twy;
    R[3] = txy + twz;       R[4] = 1 - (txx + tzz); R[5] = tyz - twx;
    R[6] = txz - twy;       R[7] = tyz + twx;       R[8] = 1 - (txx + tyy);
}

// q * v * q^-1 as v + w*uv + u x uv, uv = 2 u x v.
void rotate(const Quat& q, const double* v, double* out) {
    double uv[3] = {q.y * v[2] - q.z * v[1], q.z * v[0] - q.x * v[2], q.x * v[1] - q.y * v[0]};
    uv[0] += uv[0]; uv[1] += uv[1]; uv[2] += uv[2];
    out[0] = v[0] + q.w * uv[0] + (q.y * uv[2] - q.z * uv[1]);
    out[1] = v[1] + q.w * uv[1] + (q.z * uv[0] - q.x * uv[2]);
    out[2] = v[2] + q.w * uv[2] + (q.x * uv[1] - q.y * uv[0]);
}

Quat qmul(const Quat& a, const Quat& b) {
    Quat r;
    r.w = a.w * b.w - a.x * b.x - a.y * b.y - a.z * b.z;
    r.x = a.w * b.x + a.x * b.w + a.y * b.z - a.z * b.y;
    r.y = a.w * b.y + a.y * b.w + a.z * b.x - a.x * b.z;
    r.z = a.w * b.z + a.z * b.w + a.x * b.y - a.y * b.x;
    return r;
}

SE3 se3_from_pose12(const double* P) {
    const double R[9] = {P[0], P[1], P[2], P[4], P[5], P[6], P[8], P[9], P[10]};
    SE3 T;
    T.q = quat_from_matrix(R);
    normalize_rotation(T.q);
    T.t[0] = P[3]; T.t[1] = P[7]; T.t[2] = P[11];
    return T;
}

void pose12_from_se3(const SE3& T, double* P) {
    double R[9];
    matrix_from_quat(T.q, R);
    for (int r = 0; r < 3; ++r) {
        P[r * 4 + 0] = R[r * 3 + 0];
        P[r * 4 + 1] = R[r * 3 + 1];
        P[r * 4 + 2] = R[r * 3 + 2];
        P[r * 4 + 3] = T.t[r];
    }
}

// exp of a twist [omega; upsilon] in g2o's SE3Quat::exp semantics (see the header comment).
SE3 se3_exp(const double* d) {
    const double om[3] = {d[0], d[1], d[2]};
    const double th = std::sqrt(om[0] * om[0] + om[1] * om[1] + om[2] * om[2]);
    const double W[9] = {0, -om[2], om[1], om[2], 0, -om[0], -om[1], om[0], 0};
    double W2[9];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            W2[i * 3 + j] = W[i * 3 + 0] * W[0 * 3 + j] + W[i * 3 + 1] * W[1 * 3 + j] + W[i * 3 + 2] * W[2 * 3 + j];
    double R[9], V[9];
    if (th < 0.00001) {
        for (int k = 0; k < 9; ++k) R[k] = ((k % 4) == 0 ? 1.0 : 0.0) + W[k] + W2[k];
        for (int k = 0; k < 9; ++k) V[k] = R[k];
    } else {
        const double a = std::sin(th) / th;
        const double b = (1 - std::cos(th)) / (th * th);
        const double c = (th - std::sin(th)) / (th * th * th);
        for (int k = 0; k < 9; ++k) R[k] = ((k % 4) == 0 ? 1.0 : 0.0) + a * W[k] + b * W2[k];
        for (int k = 0; k < 9; ++k) V[k] = ((k % 4) == 0 ? 1.0 : 0.0) + b * W[k] + c * W2[k];
    }
    SE3 T;
    T.q = quat_from_matrix(R);
    normalize_rotation(T.q);
    for (int i = 0; i < 3; ++i) T.t[i] = V[i * 3 + 0] * d[3] + V[i * 3 + 1] * d[4] + V[i * 3 + 2] * d[5];
    return T;
}

SE3 compose(const SE3& a, const SE3& b) {  // g2o SE3Quat::operator*
    SE3 r;
    double rt[3];
    rotate(a.q, b.t, rt);
    for (int i = 0; i < 3; ++i) r.t[i] = a.t[i] + rt[i];
    r.q = qmul(a.q, b.q);
    normalize_rotation(r.q);
    return r;
}

// Adjugate inverse of a 3x3 matrix (row-major).
void inverse3(const double* m, double* inv) {
    const double c00 = m[4] * m[8] - m[5] * m[7];
    const double c10 = m[5] * m[6] - m[3] * m[8];
    const double c20 = m[3] * m[7] - m[4] * m[6];
    const double det = m[0] * c00 + m[1] * c10 + m[2] * c20;
    const double id = 1.0 / det;
    inv[0] = c00 * id;
    inv[1] = (m[2] * m[7] - m[1] * m[8]) * id;
    inv[2] = (m[1] * m[5] - m[2] * m[4]) * id;
    inv[3] = c10 * id;
    inv[4] = (m[0] * m[8] - m[2] * m[6]) * id;
    inv[5] = (m[2] * m[3] - m[0] * m[5]) * id;
    inv[6] = c20 * id;
    inv[7] = (m[1] * m[6] - m[0] * m[7]) * id;
    inv[8] = (m[0] * m[4] - m[1] * m[3]) * id;
}

struct EdgeLin {
    double e[2];
    double jc[12];  // 2x6 row-major
    double jp[6];   // 2x3
    double jk[4];   // 2x2 d e / d(k1,k2)
    double w;       // rho'
    double rho;     // robust chi2 of the edge
};

struct Model {
    int model;
    double fx, fy, cx, cy, k1, k2, k3 = 0.0, k4 = 0.0;
    // Kannala-Brandt 8 with the reference's own roundings (oracle_linearize_mode, mode 1): project
    // takes theta and psi through atan2f/sqrtf on float-rounded inputs and evaluates
    // r = theta + k1 theta^3 + ... with theta^5 = theta^3 theta^2, ... (KannalaBrandt8.cpp:92-107);
    // projectJac forms 3 k1, 5 k2, ... in float (int times float parameter) before widening
    // (:205-209).  The intrinsics are the float parameters nav24 keeps (Calibration.cpp:42-60).
    bool kb8_reference_rounding = false;
};

// Residual and Jacobians of one edge.  Returns false when the edge cannot be evaluated
// (it never fails; depth sign is not tested, like the reference which never calls
// isDepthPositive from GraphOptim).
void linearize_edge(const Model& m, const SE3& T, const double* X, const double* z, bool want_jac,
                    bool robust, double delta, EdgeLin& L) {
    double Xc[3];
    rotate(T.q, X, Xc);
    Xc[0] += T.t[0]; Xc[1] += T.t[1]; Xc[2] += T.t[2];
    const double x = Xc[0], y = Xc[1], zc = Xc[2];
    double u, v;
    double J[6];  // d pi / d Xc, 2x3
    double jk[4] = {0, 0, 0, 0};
    if (m.model == NAV_BA_CAM_KANNALA_BRANDT8) {
        // KannalaBrandt8::project (KannalaBrandt8.cpp:80-107) and ::projectJac (:195-226), in FP64
        // (the reference's project rounds theta and psi to float; its projectJac is FP64):
        //   theta = atan2(rho, z), r = theta + k1 theta^3 + k2 theta^5 + k3 theta^7 + k4 theta^9,
        //   (u, v) = (fx r cos psi + cx, fy r sin psi + cy) with cos psi = x / rho, sin psi = y / rho.
        // On the optical axis the limit is the pinhole projection.
        const double rho2 = x * x + y * y, rho = std::sqrt(rho2), z2 = zc * zc;
        if (rho <= 1e-9 * std::fabs(zc)) {
            u = m.fx * x / zc + m.cx;
            v = m.fy * y / zc + m.cy;
            J[0] = m.fx / zc; J[1] = 0.0; J[2] = -m.fx * x / z2;
            J[3] = 0.0; J[4] = m.fy / zc; J[5] = -m.fy * y / z2;
        } else {
            const double th = std::atan2(rho, zc);
            const double t2 = th * th, t3 = t2 * th, t4 = t2 * t2, t5 = t4 * th, t6 = t4 * t2, t7 = t6 * th,
                         t8 = t4 * t4, t9 = t8 * th;
            const double f = th + m.k1 * t3 + m.k2 * t5 + m.k3 * t7 + m.k4 * t9;
            double fd = 1.0 + 3.0 * m.k1 * t2 + 5.0 * m.k2 * t4 + 7.0 * m.k3 * t6 + 9.0 * m.k4 * t8;
            if (m.kb8_reference_rounding) {
                const float k1f = (float)m.k1, k2f = (float)m.k2, k3f = (float)m.k3, k4f = (float)m.k4;
                fd = 1.0 + (double)(3 * k1f) * t2 + (double)(5 * k2f) * t4 + (double)(7 * k3f) * t6 +
                     (double)(9 * k4f) * t8;
                const double thf = (double)atan2f(sqrtf((float)rho2), (float)zc);
                const double psi = (double)atan2f((float)y, (float)x);
                const double q2 = thf * thf, q3 = thf * q2, q5 = q3 * q2, q7 = q5 * q2, q9 = q7 * q2;
                const double r = thf + m.k1 * q3 + m.k2 * q5 + m.k3 * q7 + m.k4 * q9;
                u = m.fx * r * std::cos(psi) + m.cx;
                v = m.fy * r * std::sin(psi) + m.cy;
            } else {
                u = m.fx * f * x / rho + m.cx;
                v = m.fy * f * y / rho + m.cy;
            }
            const double rho3 = rho2 * rho, x2 = x * x, y2 = y * y;
            J[0] = m.fx * (fd * zc * x2 / (rho2 * (rho2 + z2)) + f * y2 / rho3);
            J[1] = m.fx * (fd * zc * y * x / (rho2 * (rho2 + z2)) - f * y * x / rho3);
            J[2] = -m.fx * fd * x / (rho2 + z2);
            J[3] = m.fy * (fd * zc * y * x / (rho2 * (rho2 + z2)) - f * y * x / rho3);
            J[4] = m.fy * (fd * zc * y2 / (rho2 * (rho2 + z2)) + f * x2 / rho3);
            J[5] = -m.fy * fd * y / (rho2 + z2);
        }
    } else if (m.model == NAV_BA_CAM_PINHOLE) {
        // Pinhole::project (Pinhole.cpp:30-36) and Pinhole::projectJac (Pinhole.cpp:70-80)
        u = m.fx * x / zc + m.cx;
        v = m.fy * y / zc + m.cy;
        J[0] = m.fx / zc; J[1] = 0.0; J[2] = -m.fx * x / (zc * zc);
        J[3] = 0.0; J[4] = m.fy / zc; J[5] = -m.fy * y / (zc * zc);
    } else {
        // radial factor d = 1 + k1 r^2 + k2 r^4 on normalized coordinates (no reference
        // counterpart: nav24 undistorts keypoints before BA)
        const double xn = x / zc, yn = y / zc;
        const double r2 = xn * xn + yn * yn;
        const double dd = 1.0 + m.k1 * r2 + m.k2 * r2 * r2;
        u = m.fx * dd * xn + m.cx;
        v = m.fy * dd * yn + m.cy;
        const double c = m.k1 + 2.0 * m.k2 * r2;
        const double a00 = m.fx * (dd + 2.0 * xn * xn * c), a01 = m.fx * 2.0 * xn * yn * c;
        const double a10 = m.fy * 2.0 * xn * yn * c, a11 = m.fy * (dd + 2.0 * yn * yn * c);
        const double iz = 1.0 / zc;
        J[0] = a00 * iz; J[1] = a01 * iz; J[2] = -(a00 * xn + a01 * yn) * iz;
        J[3] = a10 * iz; J[4] = a11 * iz; J[5] = -(a10 * xn + a11 * yn) * iz;
        jk[0] = -m.fx * xn * r2; jk[1] = -m.fx * xn * r2 * r2;
        jk[2] = -m.fy * yn * r2; jk[3] = -m.fy * yn * r2 * r2;
    }
    L.e[0] = z[0] - u;
    L.e[1] = z[1] - v;
    const double chi2 = L.e[0] * L.e[0] + L.e[1] * L.e[1];
    if (robust) {
        const double d2 = delta * delta;
        if (chi2 <= d2) {
            L.rho = chi2;
            L.w = 1.0;
        } else {
            const double s = std::sqrt(chi2);
            L.rho = 2 * s * delta - d2;
            L.w = delta / s;
        }
    } else {
        L.rho = chi2;
        L.w = 1.0;
    }
    if (!want_jac) return;
    for (int k = 0; k < 4; ++k) L.jk[k] = jk[k];
    double R[9];
    matrix_from_quat(T.q, R);
    double P[6];  // projectJac = -J
    for (int k = 0; k < 6; ++k) P[k] = -J[k];
    for (int r = 0; r < 2; ++r)
        for (int c = 0; c < 3; ++c)
            L.jp[r * 3 + c] = P[r * 3 + 0] * R[0 * 3 + c] + P[r * 3 + 1] * R[1 * 3 + c] + P[r * 3 + 2] * R[2 * 3 + c];
    const double D[18] = {0, zc, -y, 1, 0, 0, -zc, 0, x, 0, 1, 0, y, -x, 0, 0, 0, 1};  // SE3deriv 3x6
    for (int r = 0; r < 2; ++r)
        for (int c = 0; c < 6; ++c)
            L.jc[r * 6 + c] = P[r * 3 + 0] * D[0 * 6 + c] + P[r * 3 + 1] * D[1 * 6 + c] + P[r * 3 + 2] * D[2 * 6 + c];
}


template <class Fn>
void run_threads(int n_threads, Fn fn) {
    if (n_threads <= 1) {
        fn(0);
        return;
    }
    std::vector<std::thread> th;
    th.reserve(n_threads);
    for (int t = 0; t < n_threads; ++t) th.emplace_back(fn, t);
    for (auto& x : th) x.join();
}

inline void chunk(int n, int n_threads, int t, int& lo, int& hi) {
    const long long a = (long long)n * t / n_threads, b = (long long)n * (t + 1) / n_threads;
    lo = (int)a;
    hi = (int)b;
}

bool finite_all(const double* a, long long n) {
    for (long long i = 0; i < n; ++i)
        if (!std::isfinite(a[i])) return false;
    return true;
}

int32_t validate(const nav_ba_problem* p) {
    if (!p || p->n_cams < 0 || p->n_points < 0 || p->n_obs < 0) return NAV_BA_ERR_ARGUMENT;
    if ((p->n_cams && !p->cam_pose) || (p->n_points && !p->points) ||
        (p->n_obs && (!p->obs_uv || !p->obs_cam || !p->obs_point)))
        return NAV_BA_ERR_ARGUMENT;
    if (p->camera_model != NAV_BA_CAM_PINHOLE && p->camera_model != NAV_BA_CAM_PINHOLE_RADIAL &&
        p->camera_model != NAV_BA_CAM_KANNALA_BRANDT8)
        return NAV_BA_ERR_ARGUMENT;
    for (int o = 0; o < p->n_obs; ++o)
        if (p->obs_cam[o] < 0 || p->obs_cam[o] >= p->n_cams || p->obs_point[o] < 0 ||
            p->obs_point[o] >= p->n_points)
            return NAV_BA_ERR_ARGUMENT;
    if (!finite_all(p->cam_pose, 12LL * p->n_cams) || !finite_all(p->points, 3LL * p->n_points) ||
        !finite_all(p->obs_uv, 2LL * p->n_obs) || !finite_all(p->intrinsics, 8))
        return NAV_BA_ERR_NONFINITE_INPUT;
    return NAV_BA_OK;
}

// The BA problem as g2o would hold it after initializeOptimization().
class Solver {
public:
    const nav_ba_problem& P;
    nav_ba_options O;
    int nth;
    Model M;
    int nc, np;
    int nk = 0;  // 2 when the shared distortion pair is a free vertex
    std::vector<int32_t> cam_free, pt_free;
    int nfc = 0, nfp = 0;
    // active edges grouped by point (point-major), input order within a point
    std::vector<int32_t> pe_off, pe;
    int n_active = 0;
    std::vector<int32_t> fb;  // first structurally nonzero block column of each free-camera row
    // state
    std::vector<SE3> T;
    std::vector<double> X;
    double k[2] = {0, 0};
    // linear system at the current state
    std::vector<double> U, bc, V, bp, W, Kc, Kp;  // W per active edge (18), Kp per free point (6)
    double Kk[4] = {0, 0, 0, 0}, bk[2] = {0, 0};
    // step
    std::vector<double> dc, dp;
    double dk[2] = {0, 0};

    Solver(const nav_ba_problem& p, const nav_ba_options& o, int n_threads)
        : P(p), O(o), nth(std::max(1, n_threads)) {
        M.model = p.camera_model;
        M.fx = p.intrinsics[0]; M.fy = p.intrinsics[1];
        M.cx = p.intrinsics[2]; M.cy = p.intrinsics[3];
        M.k1 = p.intrinsics[4]; M.k2 = p.intrinsics[5];
        M.k3 = p.intrinsics[6]; M.k4 = p.intrinsics[7];
        k[0] = M.k1; k[1] = M.k2;
        nc = p.n_cams;
        np = p.n_points;
        nk = (o.optimize_distortion && p.camera_model == NAV_BA_CAM_PINHOLE_RADIAL) ? 2 : 0;
        build_graph();
        T.resize(nc);
        for (int c = 0; c < nc; ++c) T[c] = se3_from_pose12(p.cam_pose + 12LL * c);
        X.assign(p.points, p.points + 3LL * np);
    }

    bool cam_is_fixed(int c) const { return P.cam_fixed && P.cam_fixed[c]; }
    bool pt_is_fixed(int i) const { return P.point_fixed && P.point_fixed[i]; }

    void build_graph() {
        std::vector<int32_t> cnt(np + 1, 0);
        std::vector<uint8_t> act(P.n_obs, 0);
        for (int o = 0; o < P.n_obs; ++o) {
            const int c = P.obs_cam[o], i = P.obs_point[o];
            // an edge whose vertices are all fixed is not active (initializeOptimization)
            act[o] = (nk > 0) || !(cam_is_fixed(c) && pt_is_fixed(i));
            if (act[o]) cnt[i + 1]++;
        }
        pe_off.assign(np + 1, 0);
        for (int i = 0; i < np; ++i) pe_off[i + 1] = pe_off[i] + cnt[i + 1];
        pe.assign(pe_off[np], 0);
        std::vector<int32_t> fill(pe_off.begin(), pe_off.end() - 1);
        for (int o = 0; o < P.n_obs; ++o)
            if (act[o]) pe[fill[P.obs_point[o]]++] = o;
        n_active = pe_off[np];
        std::vector<uint8_t> cam_has(nc, 0);
        for (int e = 0; e < n_active; ++e) cam_has[P.obs_cam[pe[e]]] = 1;
        cam_free.assign(nc, -1);
        for (int c = 0; c < nc; ++c)
            if (!cam_is_fixed(c) && cam_has[c]) cam_free[c] = nfc++;
        pt_free.assign(np, -1);
        for (int i = 0; i < np; ++i)
            if (!pt_is_fixed(i) && pe_off[i + 1] > pe_off[i]) pt_free[i] = nfp++;
        // envelope of the reduced system (natural order of the free cameras)
        fb.assign(nfc, 0);
        for (int a = 0; a < nfc; ++a) fb[a] = a;
        for (int i = 0; i < np; ++i) {
            if (pt_free[i] < 0) continue;
            int mn = nfc;
            for (int e = pe_off[i]; e < pe_off[i + 1]; ++e) {
                const int a = cam_free[P.obs_cam[pe[e]]];
                if (a >= 0) mn = std::min(mn, a);
            }
            for (int e = pe_off[i]; e < pe_off[i + 1]; ++e) {
                const int a = cam_free[P.obs_cam[pe[e]]];
                if (a >= 0) fb[a] = std::min(fb[a], mn);
            }
        }
    }

    int dim_s() const { return 6 * nfc + nk; }

    Model model_now() const {
        Model m = M;
        m.k1 = k[0];
        m.k2 = k[1];
        return m;
    }

    // Robust chi2 of a state (SparseOptimizer::activeRobustChi2 after computeActiveErrors).
    double cost(const std::vector<SE3>& Ts, const std::vector<double>& Xs, const double* ks) const {
        Model m = M;
        m.k1 = ks[0];
        m.k2 = ks[1];
        std::vector<double> part(nth, 0.0);
        run_threads(nth, [&](int t) {
            int lo, hi;
            chunk(np, nth, t, lo, hi);
            double s = 0.0;
            EdgeLin L;
            for (int i = lo; i < hi; ++i)
                for (int e = pe_off[i]; e < pe_off[i + 1]; ++e) {
                    const int o = pe[e];
                    linearize_edge(m, Ts[P.obs_cam[o]], &Xs[3LL * i], P.obs_uv + 2LL * o, false,
                                   O.robust != 0, O.huber_delta, L);
                    s += L.rho;
                }
            part[t] = s;
        });
        double s = 0.0;
        for (double v : part) s += v;
        return s;
    }

    // BlockSolver::buildSystem: H blocks and b at the current state.
    void linearize() {
        U.assign(36LL * nfc, 0.0);
        bc.assign(6LL * nfc, 0.0);
        V.assign(9LL * nfp, 0.0);
        bp.assign(3LL * nfp, 0.0);
        W.assign(18LL * n_active, 0.0);
        Kc.assign(12LL * nfc, 0.0);
        Kp.assign(6LL * nfp, 0.0);
        std::fill(Kk, Kk + 4, 0.0);
        bk[0] = bk[1] = 0.0;
        const Model m = model_now();
        // per-thread camera-side accumulators
        std::vector<std::vector<double>> tU(nth), tb(nth), tKc(nth), tK(nth);
        run_threads(nth, [&](int t) {
            int lo, hi;
            chunk(np, nth, t, lo, hi);
            std::vector<double>& u = tU[t];
            std::vector<double>& b = tb[t];
            std::vector<double>& kc = tKc[t];
            std::vector<double>& kk = tK[t];
            u.assign(36LL * nfc, 0.0);
            b.assign(6LL * nfc, 0.0);
            kc.assign(12LL * nfc, 0.0);
            kk.assign(6, 0.0);
            EdgeLin L;
            for (int i = lo; i < hi; ++i) {
                const int fp = pt_free[i];
                for (int e = pe_off[i]; e < pe_off[i + 1]; ++e) {
                    const int o = pe[e];
                    const int c = P.obs_cam[o];
                    const int fc = cam_free[c];
                    linearize_edge(m, T[c], &X[3LL * i], P.obs_uv + 2LL * o, true, O.robust != 0,
                                   O.huber_delta, L);
                    const double w = L.w;
                    const double we0 = -w * L.e[0], we1 = -w * L.e[1];
                    if (fc >= 0) {
                        double* Ua = &u[36LL * fc];
                        for (int r = 0; r < 6; ++r)
                            for (int s = 0; s < 6; ++s)
                                Ua[r * 6 + s] += w * (L.jc[r] * L.jc[s] + L.jc[6 + r] * L.jc[6 + s]);
                        for (int r = 0; r < 6; ++r) b[6LL * fc + r] += L.jc[r] * we0 + L.jc[6 + r] * we1;
                    }
                    if (fp >= 0) {
                        double* Vp = &V[9LL * fp];
                        for (int r = 0; r < 3; ++r)
                            for (int s = 0; s < 3; ++s)
                                Vp[r * 3 + s] += w * (L.jp[r] * L.jp[s] + L.jp[3 + r] * L.jp[3 + s]);
                        for (int r = 0; r < 3; ++r) bp[3LL * fp + r] += L.jp[r] * we0 + L.jp[3 + r] * we1;
                    }
                    if (fc >= 0 && fp >= 0) {
                        double* We = &W[18LL * e];
                        for (int r = 0; r < 6; ++r)
                            for (int s = 0; s < 3; ++s)
                                We[r * 3 + s] = w * (L.jc[r] * L.jp[s] + L.jc[6 + r] * L.jp[3 + s]);
                    }
                    if (nk) {
                        // distortion vertex: rows (k1, k2)
                        for (int r = 0; r < 2; ++r) {
                            for (int s = 0; s < 2; ++s)
                                kk[r * 2 + s] += w * (L.jk[r] * L.jk[s] + L.jk[2 + r] * L.jk[2 + s]);
                            kk[4 + r] += L.jk[r] * we0 + L.jk[2 + r] * we1;
                            if (fc >= 0)
                                for (int s = 0; s < 6; ++s)
                                    kc[12LL * fc + r * 6 + s] += w * (L.jk[r] * L.jc[s] + L.jk[2 + r] * L.jc[6 + s]);
                            if (fp >= 0)
                                for (int s = 0; s < 3; ++s)
                                    Kp[6LL * fp + r * 3 + s] += w * (L.jk[r] * L.jp[s] + L.jk[2 + r] * L.jp[3 + s]);
                        }
                    }
                }
            }
        });
        for (int t = 0; t < nth; ++t) {
            for (size_t j = 0; j < U.size(); ++j) U[j] += tU[t][j];
            for (size_t j = 0; j < bc.size(); ++j) bc[j] += tb[t][j];
            for (size_t j = 0; j < Kc.size(); ++j) Kc[j] += tKc[t][j];
            for (int j = 0; j < 4; ++j) Kk[j] += tK[t][j];
            bk[0] += tK[t][4];
            bk[1] += tK[t][5];
        }
    }

    double max_diag() const {
        double m = 0.0;
        for (int a = 0; a < nfc; ++a)
            for (int r = 0; r < 6; ++r) m = std::max(m, std::fabs(U[36LL * a + r * 7]));
        for (int i = 0; i < nfp; ++i)
            for (int r = 0; r < 3; ++r) m = std::max(m, std::fabs(V[9LL * i + r * 4]));
        for (int r = 0; r < nk; ++r) m = std::max(m, std::fabs(Kk[r * 3]));
        return m;
    }

    // Reduced camera system S (dense, lower triangle filled, row-major dim x dim) and b'.
    void reduced_system(double lambda, std::vector<double>& S, std::vector<double>& bs,
                        std::vector<double>& Vinv) const {
        const int m = dim_s();
        S.assign((size_t)m * m, 0.0);
        bs.assign(m, 0.0);
        Vinv.assign(9LL * nfp, 0.0);
        for (int a = 0; a < nfc; ++a) {
            for (int r = 0; r < 6; ++r) {
                for (int s = 0; s <= r; ++s) S[(size_t)(6 * a + r) * m + 6 * a + s] = U[36LL * a + r * 6 + s];
                S[(size_t)(6 * a + r) * m + 6 * a + r] += lambda;
                bs[6 * a + r] = bc[6LL * a + r];
            }
        }
        const int kb = 6 * nfc;
        for (int r = 0; r < nk; ++r) {
            for (int a = 0; a < nfc; ++a)
                for (int s = 0; s < 6; ++s) S[(size_t)(kb + r) * m + 6 * a + s] = Kc[12LL * a + r * 6 + s];
            for (int s = 0; s <= r; ++s) S[(size_t)(kb + r) * m + kb + s] = Kk[r * 2 + s];
            S[(size_t)(kb + r) * m + kb + r] += lambda;
            bs[kb + r] = bk[r];
        }
        std::vector<std::vector<double>> tS(nth), tB(nth);
        run_threads(nth, [&](int t) {
            int lo, hi;
            chunk(np, nth, t, lo, hi);
            std::vector<double>* Sa = &S;
            std::vector<double>* Ba = &bs;
            if (nth > 1) {
                tS[t].assign((size_t)m * m, 0.0);
                tB[t].assign(m, 0.0);
                Sa = &tS[t];
                Ba = &tB[t];
            }
            std::vector<double>& SS = *Sa;
            std::vector<double>& BB = *Ba;
            std::vector<double> Y;
            for (int i = lo; i < hi; ++i) {
                const int fp = pt_free[i];
                if (fp < 0) continue;
                double Vl[9];
                for (int j = 0; j < 9; ++j) Vl[j] = V[9LL * fp + j];
                Vl[0] += lambda; Vl[4] += lambda; Vl[8] += lambda;
                double* Vi = const_cast<double*>(&Vinv[9LL * fp]);
                inverse3(Vl, Vi);
                const double* bpp = &bp[3LL * fp];
                const int e0 = pe_off[i], e1 = pe_off[i + 1];
                Y.assign(18LL * (e1 - e0), 0.0);
                for (int e = e0; e < e1; ++e) {
                    if (cam_free[P.obs_cam[pe[e]]] < 0) continue;
                    const double* We = &W[18LL * e];
                    double* Ye = &Y[18LL * (e - e0)];
                    for (int r = 0; r < 6; ++r)
                        for (int s = 0; s < 3; ++s)
                            Ye[r * 3 + s] = We[r * 3 + 0] * Vi[0 * 3 + s] + We[r * 3 + 1] * Vi[1 * 3 + s] + We[r * 3 + 2] * Vi[2 * 3 + s];
                }
                for (int e = e0; e < e1; ++e) {
                    const int a = cam_free[P.obs_cam[pe[e]]];
                    if (a < 0) continue;
                    const double* Ye = &Y[18LL * (e - e0)];
                    for (int r = 0; r < 6; ++r)
                        BB[6 * a + r] -= Ye[r * 3 + 0] * bpp[0] + Ye[r * 3 + 1] * bpp[1] + Ye[r * 3 + 2] * bpp[2];
                    for (int f = e0; f < e1; ++f) {
                        const int bcam = cam_free[P.obs_cam[pe[f]]];
                        if (bcam < 0 || bcam > a) continue;
                        const double* Wf = &W[18LL * f];
                        for (int r = 0; r < 6; ++r)
                            for (int s = 0; s < 6; ++s) {
                                if (bcam == a && s > r) continue;
                                SS[(size_t)(6 * a + r) * m + 6 * bcam + s] -=
                                    Ye[r * 3 + 0] * Wf[s * 3 + 0] + Ye[r * 3 + 1] * Wf[s * 3 + 1] + Ye[r * 3 + 2] * Wf[s * 3 + 2];
                            }
                    }
                }
                if (nk) {
                    double Z[6];  // Kp Vinv (2x3)
                    const double* K = &Kp[6LL * fp];
                    for (int r = 0; r < 2; ++r)
                        for (int s = 0; s < 3; ++s)
                            Z[r * 3 + s] = K[r * 3 + 0] * Vi[0 * 3 + s] + K[r * 3 + 1] * Vi[1 * 3 + s] + K[r * 3 + 2] * Vi[2 * 3 + s];
                    for (int r = 0; r < 2; ++r) {
                        BB[kb + r] -= Z[r * 3 + 0] * bpp[0] + Z[r * 3 + 1] * bpp[1] + Z[r * 3 + 2] * bpp[2];
                        for (int s = 0; s <= r; ++s)
                            SS[(size_t)(kb + r) * m + kb + s] -= Z[r * 3 + 0] * K[s * 3 + 0] + Z[r * 3 + 1] * K[s * 3 + 1] + Z[r * 3 + 2] * K[s * 3 + 2];
                        for (int f = e0; f < e1; ++f) {
                            const int bcam = cam_free[P.obs_cam[pe[f]]];
                            if (bcam < 0) continue;
                            const double* Wf = &W[18LL * f];
                            for (int s = 0; s < 6; ++s)
                                SS[(size_t)(kb + r) * m + 6 * bcam + s] -=
                                    Z[r * 3 + 0] * Wf[s * 3 + 0] + Z[r * 3 + 1] * Wf[s * 3 + 1] + Z[r * 3 + 2] * Wf[s * 3 + 2];
                        }
                    }
                }
            }
        });
        if (nth > 1) {
            for (int t = 0; t < nth; ++t) {
                if (tS[t].empty()) continue;
                for (size_t j = 0; j < S.size(); ++j) S[j] += tS[t][j];
                for (int j = 0; j < m; ++j) bs[j] += tB[t][j];
            }
        }
    }

    // Row envelope start of scalar row r of S.
    int row_start(int r) const {
        if (r >= 6 * nfc) return 0;
        return 6 * fb[r / 6];
    }

    // In-place LL^T inside the envelope; false when a pivot is not positive or not finite.
    bool cholesky(std::vector<double>& S) const {
        const int m = dim_s();
        for (int i = 0; i < m; ++i) {
            const int fi = row_start(i);
            double* Li = &S[(size_t)i * m];
            for (int j = fi; j < i; ++j) {
                const double* Lj = &S[(size_t)j * m];
                double s = Li[j];
                for (int kk = std::max(fi, row_start(j)); kk < j; ++kk) s -= Li[kk] * Lj[kk];
                Li[j] = s / Lj[j];
            }
            double d = Li[i];
            for (int kk = fi; kk < i; ++kk) d -= Li[kk] * Li[kk];
            if (!(d > 0.0) || !std::isfinite(d)) return false;
            Li[i] = std::sqrt(d);
        }
        return true;
    }

    void chol_solve(const std::vector<double>& L, std::vector<double>& x) const {
        const int m = dim_s();
        for (int i = 0; i < m; ++i) {
            double s = x[i];
            for (int kk = row_start(i); kk < i; ++kk) s -= L[(size_t)i * m + kk] * x[kk];
            x[i] = s / L[(size_t)i * m + i];
        }
        for (int i = m - 1; i >= 0; --i) {
            x[i] /= L[(size_t)i * m + i];
            const double xi = x[i];
            for (int kk = row_start(i); kk < i; ++kk) x[kk] -= L[(size_t)i * m + kk] * xi;
        }
    }

    // Block-Jacobi preconditioned conjugate gradients on the reduced system (NAV_BA_SOLVER_PCG):
    // preconditioner = the 6x6 camera blocks and the 2x2 distortion block of S, each factored by
    // Cholesky; x0 = 0; stop when ||r|| <= tol ||b|| (tested every 4 iterations) or after the
    // maximum number of iterations.  Returns false when a preconditioner block is not positive
    // definite.  The solution replaces bs.
    int pcg_iterations = 0;
    bool pcg_solve(const std::vector<double>& S, std::vector<double>& bs) {
        const int m = dim_s();
        auto Sij = [&](int i, int j) { return j <= i ? S[(size_t)i * m + j] : S[(size_t)j * m + i]; };
        // diagonal blocks: cameras (6x6) then the distortion pair (2x2)
        std::vector<int> bstart, bsize;
        for (int a = 0; a < nfc; ++a) { bstart.push_back(6 * a); bsize.push_back(6); }
        if (nk) { bstart.push_back(6 * nfc); bsize.push_back(nk); }
        std::vector<std::vector<double>> Lb(bstart.size());
        bool ok = true;
        for (size_t k = 0; k < bstart.size(); ++k) {
            const int s0 = bstart[k], n = bsize[k];
            std::vector<double>& L = Lb[k];
            L.assign(n * n, 0.0);
            for (int i = 0; i < n; ++i)
                for (int j = 0; j <= i; ++j) L[i * n + j] = Sij(s0 + i, s0 + j);
            for (int j = 0; j < n; ++j) {
                double d = L[j * n + j];
                for (int q = 0; q < j; ++q) d -= L[j * n + q] * L[j * n + q];
                if (!(d > 0.0) || !std::isfinite(d)) { ok = false; d = 1.0; }
                L[j * n + j] = std::sqrt(d);
                for (int i = j + 1; i < n; ++i) {
                    double v = L[i * n + j];
                    for (int q = 0; q < j; ++q) v -= L[i * n + q] * L[j * n + q];
                    L[i * n + j] = v / L[j * n + j];
                }
            }
        }
        auto precond = [&](const std::vector<double>& r, std::vector<double>& z) {
            z.assign(m, 0.0);
            for (size_t k = 0; k < bstart.size(); ++k) {
                const int s0 = bstart[k], n = bsize[k];
                const std::vector<double>& L = Lb[k];
                double v[6];
                for (int i = 0; i < n; ++i) {
                    double t = r[s0 + i];
                    for (int q = 0; q < i; ++q) t -= L[i * n + q] * v[q];
                    v[i] = t / L[i * n + i];
                }
                for (int i = n - 1; i >= 0; --i) {
                    double t = v[i];
                    for (int q = i + 1; q < n; ++q) t -= L[q * n + i] * v[q];
                    v[i] = t / L[i * n + i];
                }
                for (int i = 0; i < n; ++i) z[s0 + i] = v[i];
            }
        };
        std::vector<double> x(m, 0.0), r = bs, z, p, q(m);
        precond(r, z);
        p = z;
        double rz = 0.0, rr = 0.0;
        for (int i = 0; i < m; ++i) { rz += r[i] * z[i]; rr += r[i] * r[i]; }
        const double bb = rr;
        const double tol2 = O.pcg_tolerance * O.pcg_tolerance;
        int it = 0;
        for (; it < O.pcg_max_iterations; ++it) {
            if (it % 4 == 0 && !(rr > tol2 * bb)) break;
            for (int i = 0; i < m; ++i) {
                double t = 0.0;
                for (int j = 0; j < m; ++j) t += Sij(i, j) * p[j];
                q[i] = t;
            }
            double pq = 0.0;
            for (int i = 0; i < m; ++i) pq += p[i] * q[i];
            const double alpha = pq != 0.0 ? rz / pq : 0.0;
            for (int i = 0; i < m; ++i) { x[i] += alpha * p[i]; r[i] -= alpha * q[i]; }
            precond(r, z);
            double rzn = 0.0;
            rr = 0.0;
            for (int i = 0; i < m; ++i) { rzn += r[i] * z[i]; rr += r[i] * r[i]; }
            const double beta = rz != 0.0 ? rzn / rz : 0.0;
            for (int i = 0; i < m; ++i) p[i] = z[i] + beta * p[i];
            rz = rzn;
        }
        pcg_iterations += it;
        bs = x;
        return ok;
    }

    // ---- block-sparse reduced system (the PCG solver): only the nonzero 6x6 blocks of S ----------
    // Lower blocks (a >= b) of the free cameras that share a free point, by block row, in increasing
    // column order; each block is 36 values, row-major (diagonal blocks held whole).  Built once.
    std::vector<int32_t> srow_off, scol;
    void build_block_pattern() {
        if (!srow_off.empty() || nfc == 0) return;
        std::vector<std::vector<int32_t>> rows(nfc);
        for (int a = 0; a < nfc; ++a) rows[a].push_back(a);
        std::vector<int32_t> cams;
        for (int i = 0; i < np; ++i) {
            if (pt_free[i] < 0) continue;
            cams.clear();
            for (int e = pe_off[i]; e < pe_off[i + 1]; ++e) {
                const int a = cam_free[P.obs_cam[pe[e]]];
                if (a >= 0) cams.push_back(a);
            }
            for (int x : cams)
                for (int y : cams)
                    if (y < x) rows[x].push_back(y);
        }
        srow_off.assign(nfc + 1, 0);
        for (int a = 0; a < nfc; ++a) {
            std::sort(rows[a].begin(), rows[a].end());
            rows[a].erase(std::unique(rows[a].begin(), rows[a].end()), rows[a].end());
            srow_off[a + 1] = srow_off[a] + (int32_t)rows[a].size();
        }
        scol.reserve(srow_off[nfc]);
        for (int a = 0; a < nfc; ++a) scol.insert(scol.end(), rows[a].begin(), rows[a].end());
    }
    int block_of(int a, int b) const {
        const int32_t* lo = scol.data() + srow_off[a];
        const int32_t* hi = scol.data() + srow_off[a + 1];
        return (int)(std::lower_bound(lo, hi, b) - scol.data());
    }

    // The reduced system of reduced_system() in block form: Sb [blocks][36] (lower blocks, the
    // diagonal ones whole), the distortion rows SK [nk][6 nfc + nk] (dense) and b'.  Per-thread
    // block copies summed in thread order.
    void reduced_system_blocks(double lambda, std::vector<double>& Sb, std::vector<double>& SK,
                               std::vector<double>& bs, std::vector<double>& Vinv) const {
        const int m = dim_s(), kb = 6 * nfc, nb = srow_off.empty() ? 0 : srow_off[nfc];
        Vinv.assign(9LL * nfp, 0.0);
        Sb.assign(36LL * nb, 0.0);
        SK.assign((size_t)nk * m, 0.0);
        bs.assign(m, 0.0);
        for (int a = 0; a < nfc; ++a) {
            double* B = &Sb[36LL * block_of(a, a)];
            for (int r = 0; r < 6; ++r) {
                for (int s = 0; s < 6; ++s) B[r * 6 + s] = U[36LL * a + r * 6 + s];
                B[r * 6 + r] += lambda;
                bs[6 * a + r] = bc[6LL * a + r];
            }
        }
        for (int r = 0; r < nk; ++r) {
            for (int a = 0; a < nfc; ++a)
                for (int s = 0; s < 6; ++s) SK[(size_t)r * m + 6 * a + s] = Kc[12LL * a + r * 6 + s];
            for (int s = 0; s < nk; ++s) SK[(size_t)r * m + kb + s] = Kk[r * 2 + s];
            SK[(size_t)r * m + kb + r] += lambda;
            bs[kb + r] = bk[r];
        }
        std::vector<std::vector<double>> tS(nth), tK(nth), tB(nth);
        run_threads(nth, [&](int t) {
            int lo, hi;
            chunk(np, nth, t, lo, hi);
            std::vector<double>& SS = tS[t];
            std::vector<double>& KK = tK[t];
            std::vector<double>& BB = tB[t];
            SS.assign(36LL * nb, 0.0);
            KK.assign((size_t)nk * m, 0.0);
            BB.assign(m, 0.0);
            std::vector<double> Y;
            for (int i = lo; i < hi; ++i) {
                const int fp = pt_free[i];
                if (fp < 0) continue;
                double Vl[9];
                double* Vi = const_cast<double*>(&Vinv[9LL * fp]);
                for (int j = 0; j < 9; ++j) Vl[j] = V[9LL * fp + j];
                Vl[0] += lambda; Vl[4] += lambda; Vl[8] += lambda;
                inverse3(Vl, Vi);
                const double* bpp = &bp[3LL * fp];
                const int e0 = pe_off[i], e1 = pe_off[i + 1];
                Y.assign(18LL * (e1 - e0), 0.0);
                for (int e = e0; e < e1; ++e) {
                    if (cam_free[P.obs_cam[pe[e]]] < 0) continue;
                    const double* We = &W[18LL * e];
                    double* Ye = &Y[18LL * (e - e0)];
                    for (int r = 0; r < 6; ++r)
                        for (int s = 0; s < 3; ++s)
                            Ye[r * 3 + s] = We[r * 3 + 0] * Vi[0 * 3 + s] + We[r * 3 + 1] * Vi[1 * 3 + s] + We[r * 3 + 2] * Vi[2 * 3 + s];
                }
                for (int e = e0; e < e1; ++e) {
                    const int a = cam_free[P.obs_cam[pe[e]]];
                    if (a < 0) continue;
                    const double* Ye = &Y[18LL * (e - e0)];
                    for (int r = 0; r < 6; ++r)
                        BB[6 * a + r] -= Ye[r * 3 + 0] * bpp[0] + Ye[r * 3 + 1] * bpp[1] + Ye[r * 3 + 2] * bpp[2];
                    for (int f = e0; f < e1; ++f) {
                        const int b = cam_free[P.obs_cam[pe[f]]];
                        if (b < 0 || b > a) continue;
                        const double* Wf = &W[18LL * f];
                        double* Bk = &SS[36LL * block_of(a, b)];
                        for (int r = 0; r < 6; ++r)
                            for (int s = 0; s < 6; ++s) {
                                const double v = Ye[r * 3 + 0] * Wf[s * 3 + 0] + Ye[r * 3 + 1] * Wf[s * 3 + 1] + Ye[r * 3 + 2] * Wf[s * 3 + 2];
                                Bk[r * 6 + s] -= v;
                            }
                    }
                }
                if (nk) {
                    double Z[6];
                    const double* K = &Kp[6LL * fp];
                    for (int r = 0; r < 2; ++r)
                        for (int s = 0; s < 3; ++s)
                            Z[r * 3 + s] = K[r * 3 + 0] * Vi[0 * 3 + s] + K[r * 3 + 1] * Vi[1 * 3 + s] + K[r * 3 + 2] * Vi[2 * 3 + s];
                    for (int r = 0; r < 2; ++r) {
                        BB[kb + r] -= Z[r * 3 + 0] * bpp[0] + Z[r * 3 + 1] * bpp[1] + Z[r * 3 + 2] * bpp[2];
                        for (int s = 0; s < 2; ++s)
                            KK[(size_t)r * m + kb + s] -= Z[r * 3 + 0] * K[s * 3 + 0] + Z[r * 3 + 1] * K[s * 3 + 1] + Z[r * 3 + 2] * K[s * 3 + 2];
                        for (int f = e0; f < e1; ++f) {
                            const int b = cam_free[P.obs_cam[pe[f]]];
                            if (b < 0) continue;
                            const double* Wf = &W[18LL * f];
                            for (int s = 0; s < 6; ++s)
                                KK[(size_t)r * m + 6 * b + s] -= Z[r * 3 + 0] * Wf[s * 3 + 0] + Z[r * 3 + 1] * Wf[s * 3 + 1] + Z[r * 3 + 2] * Wf[s * 3 + 2];
                        }
                    }
                }
            }
        });
        for (int t = 0; t < nth; ++t) {
            for (size_t j = 0; j < Sb.size(); ++j) Sb[j] += tS[t][j];
            for (size_t j = 0; j < SK.size(); ++j) SK[j] += tK[t][j];
            for (int j = 0; j < m; ++j) bs[j] += tB[t][j];
        }
    }

    // pcg_solve over the block form: the same preconditioner (the camera blocks and the distortion
    // block, each factored by Cholesky), iteration and stopping rule; S p from the blocks.
    bool pcg_solve_blocks(const std::vector<double>& Sb, const std::vector<double>& SK, std::vector<double>& bs) {
        const int m = dim_s(), kb = 6 * nfc;
        std::vector<std::vector<double>> Lb(nfc + (nk ? 1 : 0));
        bool ok = true;
        auto factor = [&](std::vector<double>& L, int n) {
            for (int j = 0; j < n; ++j) {
                double d = L[j * n + j];
                for (int q = 0; q < j; ++q) d -= L[j * n + q] * L[j * n + q];
                if (!(d > 0.0) || !std::isfinite(d)) { ok = false; d = 1.0; }
                L[j * n + j] = std::sqrt(d);
                for (int i = j + 1; i < n; ++i) {
                    double v = L[i * n + j];
                    for (int q = 0; q < j; ++q) v -= L[i * n + q] * L[j * n + q];
                    L[i * n + j] = v / L[j * n + j];
                }
            }
        };
        for (int a = 0; a < nfc; ++a) {
            Lb[a].assign(Sb.begin() + 36LL * block_of(a, a), Sb.begin() + 36LL * block_of(a, a) + 36);
            factor(Lb[a], 6);
        }
        if (nk) {
            Lb[nfc].assign(4, 0.0);
            for (int r = 0; r < 2; ++r)
                for (int s = 0; s < 2; ++s) Lb[nfc][r * 2 + s] = SK[(size_t)r * m + kb + s];
            factor(Lb[nfc], 2);
        }
        auto precond = [&](const std::vector<double>& r, std::vector<double>& z) {
            z.assign(m, 0.0);
            for (size_t k = 0; k < Lb.size(); ++k) {
                const int s0 = (int)k < nfc ? 6 * (int)k : kb, n = (int)k < nfc ? 6 : nk;
                const std::vector<double>& L = Lb[k];
                double v[6];
                for (int i = 0; i < n; ++i) {
                    double t = r[s0 + i];
                    for (int q = 0; q < i; ++q) t -= L[i * n + q] * v[q];
                    v[i] = t / L[i * n + i];
                }
                for (int i = n - 1; i >= 0; --i) {
                    double t = v[i];
                    for (int q = i + 1; q < n; ++q) t -= L[q * n + i] * v[q];
                    v[i] = t / L[i * n + i];
                }
                for (int i = 0; i < n; ++i) z[s0 + i] = v[i];
            }
        };
        auto matvec = [&](const std::vector<double>& p, std::vector<double>& q) {
            std::fill(q.begin(), q.end(), 0.0);
            for (int a = 0; a < nfc; ++a)
                for (int k = srow_off[a]; k < srow_off[a + 1]; ++k) {
                    const int b = scol[k];
                    const double* B = &Sb[36LL * k];
                    for (int r = 0; r < 6; ++r) {
                        double t = 0.0;
                        for (int s = 0; s < 6; ++s) t += B[r * 6 + s] * p[6 * b + s];
                        q[6 * a + r] += t;
                    }
                    if (b != a)
                        for (int s = 0; s < 6; ++s) {
                            double t = 0.0;
                            for (int r = 0; r < 6; ++r) t += B[r * 6 + s] * p[6 * a + r];
                            q[6 * b + s] += t;
                        }
                }
            for (int r = 0; r < nk; ++r) {
                double t = 0.0;
                for (int j = 0; j < m; ++j) t += SK[(size_t)r * m + j] * p[j];
                q[kb + r] += t;
                for (int j = 0; j < kb; ++j) q[j] += SK[(size_t)r * m + j] * p[kb + r];
            }
        };
        std::vector<double> x(m, 0.0), r = bs, z, p, q(m);
        precond(r, z);
        p = z;
        double rz = 0.0, rr = 0.0;
        for (int i = 0; i < m; ++i) { rz += r[i] * z[i]; rr += r[i] * r[i]; }
        const double bb = rr;
        const double tol2 = O.pcg_tolerance * O.pcg_tolerance;
        int it = 0;
        for (; it < O.pcg_max_iterations; ++it) {
            if (it % 4 == 0 && !(rr > tol2 * bb)) break;
            matvec(p, q);
            double pq = 0.0;
            for (int i = 0; i < m; ++i) pq += p[i] * q[i];
            const double alpha = pq != 0.0 ? rz / pq : 0.0;
            for (int i = 0; i < m; ++i) { x[i] += alpha * p[i]; r[i] -= alpha * q[i]; }
            precond(r, z);
            double rzn = 0.0;
            rr = 0.0;
            for (int i = 0; i < m; ++i) { rzn += r[i] * z[i]; rr += r[i] * r[i]; }
            const double beta = rz != 0.0 ? rzn / rz : 0.0;
            for (int i = 0; i < m; ++i) p[i] = z[i] + beta * p[i];
            rz = rzn;
        }
        pcg_iterations += it;
        bs = x;
        return ok;
    }

    // BlockSolver::solve with the damping applied (setLambda .. restoreDiagonal).
    bool compute_step(double lambda) {
        std::vector<double> S, bs, Vinv;
        bool ok;
        if (O.solver == NAV_BA_SOLVER_PCG) {
            build_block_pattern();
            std::vector<double> SK;
            reduced_system_blocks(lambda, S, SK, bs, Vinv);
            ok = pcg_solve_blocks(S, SK, bs);
            if (!ok) std::fill(bs.begin(), bs.end(), 0.0);
        } else {
            reduced_system(lambda, S, bs, Vinv);
            ok = cholesky(S);
            if (ok) chol_solve(S, bs);
            else std::fill(bs.begin(), bs.end(), 0.0);
        }
        const int m = dim_s();
        dc.assign(6LL * nfc, 0.0);
        for (int j = 0; j < 6 * nfc; ++j) dc[j] = bs[j];
        dk[0] = nk ? bs[m - 2] : 0.0;
        dk[1] = nk ? bs[m - 1] : 0.0;
        dp.assign(3LL * nfp, 0.0);
        run_threads(nth, [&](int t) {
            int lo, hi;
            chunk(np, nth, t, lo, hi);
            for (int i = lo; i < hi; ++i) {
                const int fp = pt_free[i];
                if (fp < 0) continue;
                double c[3] = {bp[3LL * fp], bp[3LL * fp + 1], bp[3LL * fp + 2]};
                for (int e = pe_off[i]; e < pe_off[i + 1]; ++e) {
                    const int a = cam_free[P.obs_cam[pe[e]]];
                    if (a < 0) continue;
                    const double* We = &W[18LL * e];
                    for (int s = 0; s < 3; ++s)
                        for (int r = 0; r < 6; ++r) c[s] -= We[r * 3 + s] * dc[6LL * a + r];
                }
                if (nk) {
                    const double* K = &Kp[6LL * fp];
                    for (int s = 0; s < 3; ++s) c[s] -= K[s] * dk[0] + K[3 + s] * dk[1];
                }
                const double* Vi = &Vinv[9LL * fp];
                for (int r = 0; r < 3; ++r) dp[3LL * fp + r] = Vi[r * 3 + 0] * c[0] + Vi[r * 3 + 1] * c[1] + Vi[r * 3 + 2] * c[2];
            }
        });
        return ok;
    }

    // OptimizationAlgorithmLevenberg::computeScale (without the +1e-3).
    double step_scale(double lambda) const {
        double s = 0.0;
        for (int j = 0; j < 6 * nfc; ++j) s += dc[j] * (lambda * dc[j] + bc[j]);
        for (int j = 0; j < 3 * nfp; ++j) s += dp[j] * (lambda * dp[j] + bp[j]);
        for (int j = 0; j < nk; ++j) s += dk[j] * (lambda * dk[j] + bk[j]);
        return s;
    }

    void apply_step(std::vector<SE3>& Tn, std::vector<double>& Xn, double* kn) const {
        Tn = T;
        Xn = X;
        for (int c = 0; c < nc; ++c) {
            const int a = cam_free[c];
            if (a < 0) continue;
            Tn[c] = compose(se3_exp(&dc[6LL * a]), T[c]);
        }
        for (int i = 0; i < np; ++i) {
            const int fp = pt_free[i];
            if (fp < 0) continue;
            for (int r = 0; r < 3; ++r) Xn[3LL * i + r] += dp[3LL * fp + r];
        }
        kn[0] = k[0] + dk[0];
        kn[1] = k[1] + dk[1];
    }

    // record != null: the damping of every accepted step is appended.  replay != null: those
    // steps are applied unconditionally instead of the LM control (the frozen-schedule function
    // that the product's nav_ba_vjp differentiates).
    int32_t solve(nav_ba_result* res, std::vector<double>* record = nullptr, const std::vector<double>* replay = nullptr) {
        const int iters = O.iterations;
        double chi = cost(T, X, k);
        res->initial_cost = chi;
        res->n_active_edges = n_active;
        res->n_free_cams = nfc;
        res->n_free_points = nfp;
        if (res->cost_trace) res->cost_trace[0] = chi;
        if (!std::isfinite(chi)) return NAV_BA_ERR_NONFINITE_COST;
        res->termination = NAV_BA_TERM_ITERATIONS;
        if (nfc + nfp + nk == 0) {
            res->termination = NAV_BA_TERM_NOTHING_TO_DO;
            res->final_cost = chi;
            return NAV_BA_OK;
        }
        double lambda = 0.0, nu = 2.0;
        int it = 0;
        int acc = 0, rej = 0;
        if (replay) {
            for (const double lam : *replay) {
                linearize();
                if (!compute_step(lam)) return NAV_BA_ERR_UNSUPPORTED;
                std::vector<SE3> Tn;
                std::vector<double> Xn;
                double kn[2];
                apply_step(Tn, Xn, kn);
                T.swap(Tn);
                X.swap(Xn);
                k[0] = kn[0];
                k[1] = kn[1];
                chi = cost(T, X, k);
                ++it;
                if (res->cost_trace) res->cost_trace[it] = chi;
                lambda = lam;
            }
            res->iterations_done = it;
            res->trials_accepted = it;
            res->trials_rejected = 0;
            res->final_cost = chi;
            res->final_lambda = lambda;
            return NAV_BA_OK;
        }
        for (; it < iters; ++it) {
            linearize();
            if (it == 0) {
                lambda = O.initial_lambda > 0 ? O.initial_lambda : O.tau * max_diag();
                nu = 2.0;
            }
            double rho = 0.0;
            int q = 0;
            std::vector<SE3> Tn;
            std::vector<double> Xn;
            double kn[2];
            do {
                const bool ok = compute_step(lambda);
                apply_step(Tn, Xn, kn);
                double chi_new = cost(Tn, Xn, kn);
                if (!ok) chi_new = std::numeric_limits<double>::max();
                rho = chi - chi_new;
                double scale = step_scale(lambda);
                scale += 1e-3;
                rho /= scale;
                if (rho > 0 && std::isfinite(chi_new)) {
                    if (record) record->push_back(lambda);
                    double alpha = 1.0 - std::pow(2 * rho - 1, 3);
                    alpha = std::min(alpha, 2.0 / 3.0);
                    const double sf = std::max(1.0 / 3.0, alpha);
                    lambda *= sf;
                    nu = 2;
                    chi = chi_new;
                    T.swap(Tn);
                    X.swap(Xn);
                    k[0] = kn[0];
                    k[1] = kn[1];
                    ++acc;
                } else {
                    lambda *= nu;
                    nu *= 2;
                    ++rej;
                }
                ++q;
            } while (rho < 0 && q < O.max_trials);
            if (res->cost_trace) res->cost_trace[it + 1] = chi;
            if (q == O.max_trials) { res->termination = NAV_BA_TERM_TRIALS_EXHAUSTED; ++it; break; }
            if (rho == 0) { res->termination = NAV_BA_TERM_ZERO_GAIN; ++it; break; }
            if (!std::isfinite(lambda)) { res->termination = NAV_BA_TERM_LAMBDA_NONFINITE; ++it; break; }
        }
        res->iterations_done = it;
        res->pcg_iterations_total = pcg_iterations;
        res->trials_accepted = acc;
        res->trials_rejected = rej;
        res->final_cost = chi;
        res->final_lambda = lambda;
        return NAV_BA_OK;
    }

    // Active edges for which EdgeSE3ProjectXYZ::isDepthPositive (OptimizableTypes.hpp:109-113) is
    // false at the current state: T.map(X)(2) <= 0.
    int depth_nonpositive() const {
        int n = 0;
        for (int i = 0; i < np; ++i)
            for (int e = pe_off[i]; e < pe_off[i + 1]; ++e) {
                double Xc[3];
                const SE3& Tc = T[P.obs_cam[pe[e]]];
                rotate(Tc.q, &X[3LL * i], Xc);
                n += Xc[2] + Tc.t[2] <= 0.0 ? 1 : 0;
            }
        return n;
    }

    void write_outputs(nav_ba_result* res) const {
        res->n_depth_nonpositive = depth_nonpositive();
        if (res->cam_pose_out)
            for (int c = 0; c < nc; ++c) pose12_from_se3(T[c], res->cam_pose_out + 12LL * c);
        if (res->points_out) std::memcpy(res->points_out, X.data(), sizeof(double) * 3 * np);
        if (res->intrinsics_out) {
            std::memcpy(res->intrinsics_out, P.intrinsics, sizeof(double) * 8);
            res->intrinsics_out[4] = k[0];
            res->intrinsics_out[5] = k[1];
        }
    }
};

int count_schur_blocks(const Solver& s) {
    std::vector<std::vector<int>> rows(s.nfc);
    for (int i = 0; i < s.np; ++i) {
        if (s.pt_free[i] < 0) continue;
        for (int e = s.pe_off[i]; e < s.pe_off[i + 1]; ++e) {
            const int a = s.cam_free[s.P.obs_cam[s.pe[e]]];
            if (a < 0) continue;
            for (int f = s.pe_off[i]; f < s.pe_off[i + 1]; ++f) {
                const int b = s.cam_free[s.P.obs_cam[s.pe[f]]];
                if (b >= 0 && b <= a) rows[a].push_back(b);
            }
        }
    }
    int n = 0;
    for (int a = 0; a < s.nfc; ++a) {
        rows[a].push_back(a);
        std::sort(rows[a].begin(), rows[a].end());
        n += (int)(std::unique(rows[a].begin(), rows[a].end()) - rows[a].begin());
    }
    return n;
}

}  // namespace

extern "C" int32_t oracle_solve_schedule(const nav_ba_problem* p, const nav_ba_options* o, nav_ba_result* r,
                                         int32_t n_threads, nav_ba_schedule* sched) {
    if (!o || !r) return NAV_BA_ERR_ARGUMENT;
    int32_t st = validate(p);
    if (st != NAV_BA_OK) return st;
    if (o->iterations < 0 || o->max_trials < 1 || (o->robust && !(o->huber_delta > 0)))
        return NAV_BA_ERR_ARGUMENT;
    Solver s(*p, *o, n_threads);
    if (p->n_cams == 0 || s.n_active == 0) {
        // nav24 returns without touching anything when there is no pose or no point vertex
        if (r->cam_pose_out) std::memcpy(r->cam_pose_out, p->cam_pose, sizeof(double) * 12 * p->n_cams);
        if (r->points_out) std::memcpy(r->points_out, p->points, sizeof(double) * 3 * p->n_points);
        if (r->intrinsics_out) std::memcpy(r->intrinsics_out, p->intrinsics, sizeof(double) * 8);
        r->termination = NAV_BA_TERM_NOTHING_TO_DO;
        r->iterations_done = 0;
        return NAV_BA_EMPTY;
    }
    std::vector<double> rec, rep;
    if (sched && sched->replay) {
        if (sched->n_steps < 0 || sched->n_steps > NAV_BA_VJP_MAX_STEPS) return NAV_BA_ERR_ARGUMENT;
        rep.assign(sched->lambda, sched->lambda + sched->n_steps);
    }
    st = s.solve(r, sched && !sched->replay ? &rec : nullptr, sched && sched->replay ? &rep : nullptr);
    if (st != NAV_BA_OK) return st;
    if (sched && !sched->replay) {
        sched->n_steps = (int32_t)rec.size();
        for (size_t i = 0; i < rec.size() && i < NAV_BA_VJP_MAX_STEPS; ++i) sched->lambda[i] = rec[i];
    }
    r->n_schur_blocks = count_schur_blocks(s);
    s.write_outputs(r);
    return NAV_BA_OK;
}

extern "C" int32_t oracle_solve(const nav_ba_problem* p, const nav_ba_options* o, nav_ba_result* r,
                                int32_t n_threads) {
    return oracle_solve_schedule(p, o, r, n_threads, nullptr);
}

extern "C" int32_t oracle_linearize(const nav_ba_problem* p, const nav_ba_options* o, double* e,
                                    double* jc, double* jp, double* w) {
    return oracle_linearize_mode(p, o, 0, e, jc, jp, w);
}

extern "C" int32_t oracle_linearize_mode(const nav_ba_problem* p, const nav_ba_options* o, int32_t mode,
                                         double* e, double* jc, double* jp, double* w) {
    if (!o || mode < 0 || mode > 1) return NAV_BA_ERR_ARGUMENT;
    int32_t st = validate(p);
    if (st != NAV_BA_OK) return st;
    Model m;
    m.kb8_reference_rounding = mode == 1;
    m.model = p->camera_model;
    m.fx = p->intrinsics[0]; m.fy = p->intrinsics[1]; m.cx = p->intrinsics[2]; m.cy = p->intrinsics[3];
    m.k1 = p->intrinsics[4]; m.k2 = p->intrinsics[5];
    m.k3 = p->intrinsics[6]; m.k4 = p->intrinsics[7];
    EdgeLin L;
    for (int k = 0; k < p->n_obs; ++k) {
        const SE3 T = se3_from_pose12(p->cam_pose + 12LL * p->obs_cam[k]);
        linearize_edge(m, T, p->points + 3LL * p->obs_point[k], p->obs_uv + 2LL * k, true,
                       o->robust != 0, o->huber_delta, L);
        if (e) { e[2LL * k] = L.e[0]; e[2LL * k + 1] = L.e[1]; }
        if (jc) std::memcpy(jc + 12LL * k, L.jc, sizeof(L.jc));
        if (jp) std::memcpy(jp + 6LL * k, L.jp, sizeof(L.jp));
        if (w) w[k] = L.w;
    }
    return NAV_BA_OK;
}

extern "C" int32_t oracle_distortion_jacobian(const nav_ba_problem* p, double* jk) {
    int32_t st = validate(p);
    if (st != NAV_BA_OK) return st;
    Model m;
    m.model = p->camera_model;
    m.fx = p->intrinsics[0]; m.fy = p->intrinsics[1]; m.cx = p->intrinsics[2]; m.cy = p->intrinsics[3];
    m.k1 = p->intrinsics[4]; m.k2 = p->intrinsics[5];
    m.k3 = p->intrinsics[6]; m.k4 = p->intrinsics[7];
    EdgeLin L;
    for (int k = 0; k < p->n_obs; ++k) {
        const SE3 T = se3_from_pose12(p->cam_pose + 12LL * p->obs_cam[k]);
        linearize_edge(m, T, p->points + 3LL * p->obs_point[k], p->obs_uv + 2LL * k, true, false, 1.0, L);
        std::memcpy(jk + 4LL * k, L.jk, sizeof(L.jk));
    }
    return NAV_BA_OK;
}

extern "C" int32_t oracle_reduced_system(const nav_ba_problem* p, const nav_ba_options* o,
                                         double lambda, int32_t capacity_free, int32_t* n_free,
                                         double* s, double* b, int32_t* cam_index) {
    if (!o || !n_free) return NAV_BA_ERR_ARGUMENT;
    int32_t st = validate(p);
    if (st != NAV_BA_OK) return st;
    Solver sv(*p, *o, 1);
    *n_free = sv.nfc;
    if (cam_index) std::memcpy(cam_index, sv.cam_free.data(), sizeof(int32_t) * p->n_cams);
    if (capacity_free < sv.nfc || !s || !b) return NAV_BA_OK;
    sv.linearize();
    std::vector<double> S, bs, Vinv;
    sv.reduced_system(lambda, S, bs, Vinv);
    const int m = sv.dim_s();
    const int n = 6 * sv.nfc;
    for (int i = 0; i < n; ++i) {
        b[i] = bs[i];
        for (int j = 0; j < n; ++j) s[(size_t)i * n + j] = (j <= i) ? S[(size_t)i * m + j] : S[(size_t)j * m + i];
    }
    return NAV_BA_OK;
}

extern "C" int32_t oracle_cost(const nav_ba_problem* p, const nav_ba_options* o, double* cost) {
    if (!o || !cost) return NAV_BA_ERR_ARGUMENT;
    int32_t st = validate(p);
    if (st != NAV_BA_OK) return st;
    Solver sv(*p, *o, 1);
    *cost = sv.cost(sv.T, sv.X, sv.k);
    return NAV_BA_OK;
}

extern "C" void oracle_se3_update(const double* pose12, const double* delta6, double* out12) {
    const SE3 T = se3_from_pose12(pose12);
    pose12_from_se3(compose(se3_exp(delta6), T), out12);
}

extern "C" void oracle_pose_roundtrip(const double* pose12, double* out12) {
    pose12_from_se3(se3_from_pose12(pose12), out12);
}
