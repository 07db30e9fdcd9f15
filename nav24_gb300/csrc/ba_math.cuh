// ba_math.cuh - device/host math of the BA edge and the SE(3) vertex.
//
// Edge: nav24's EdgeSE3ProjectXYZ (core/dataTypes/optimization/OptimizableTypes.hpp:92-118,
// OptimizableTypes.cpp:140-161): e = z - pi(T X), J_point = -Jpi R, J_pose = -Jpi [-[Xc]x | I]
// with the pinhole pi of core/sensor/camera/models/Pinhole.cpp:30-36,70-80.
// Vertex update: g2o VertexSE3Expmap (T <- exp(d) T, d = [omega; upsilon]) as used through
// nav24's MyVertexSE3Expmap (OptimizableTypes.hpp:221-227); point update X += d
// (MyVertexSBAPointXYZ, :229-235).
#pragma once

#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#define NAVBA_HD __host__ __device__ __forceinline__

namespace navba {

struct Intr {
    double fx, fy, cx, cy, k1, k2, k3, k4;
    int model;  // 0 pinhole, 1 pinhole + radial (k1, k2), 2 Kannala-Brandt (k1..k4)
    float f[8];  // the same eight values rounded to float once (the mixed form's arithmetic)
};

// Intrinsics from the 8 values of nav_ba_problem::intrinsics and the camera model.
NAVBA_HD Intr make_intr(const double* k8, int model) {
    Intr in{k8[0], k8[1], k8[2], k8[3], k8[4], k8[5], k8[6], k8[7], model, {}};
    for (int k = 0; k < 8; ++k) in.f[k] = (float)k8[k];
    return in;
}

// New radial coefficients (k1, k2), in both precisions.
NAVBA_HD void set_radial(Intr& in, double k1, double k2) {
    in.k1 = k1;
    in.k2 = k2;
    in.f[4] = (float)k1;
    in.f[5] = (float)k2;
}

// The intrinsics in precision Real: the FP64 values, or their float copies (no conversion per use).
template <class Real>
struct IntrV {
    Real fx, fy, cx, cy, k1, k2, k3, k4;
};
template <class Real>
NAVBA_HD IntrV<Real> intr_in(const Intr& in) {
    if constexpr (sizeof(Real) == 4)
        return IntrV<Real>{in.f[0], in.f[1], in.f[2], in.f[3], in.f[4], in.f[5], in.f[6], in.f[7]};
    else
        return IntrV<Real>{in.fx, in.fy, in.cx, in.cy, in.k1, in.k2, in.k3, in.k4};
}

// ---- quaternions (x, y, z, w), unit, w >= 0 ---------------------------------------------

NAVBA_HD void q_normalize(double* q) {
    if (q[3] < 0) {
        q[0] = -q[0]; q[1] = -q[1]; q[2] = -q[2]; q[3] = -q[3];
    }
    const double n = sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
    q[0] /= n; q[1] /= n; q[2] /= n; q[3] /= n;
}

// Shepperd's method: quaternion of a row-major rotation matrix.
NAVBA_HD void q_from_rot(const double* R, double* q) {
    const double tr = R[0] + R[4] + R[8];
    if (tr > 0.0) {
        double s = sqrt(tr + 1.0);
        q[3] = 0.5 * s;
        s = 0.5 / s;
        q[0] = (R[7] - R[5]) * s;
        q[1] = (R[2] - R[6]) * s;
        q[2] = (R[3] - R[1]) * s;
    } else {
        int i = 0;
        if (R[4] > R[0]) i = 1;
        if (R[8] > R[i * 4]) i = 2;
        const int j = (i + 1) % 3, k = (j + 1) % 3;
        double s = sqrt(R[i * 4] - R[j * 4] - R[k * 4] + 1.0);
        q[i] = 0.5 * s;
        s = 0.5 / s;
        q[3] = (R[k * 3 + j] - R[j * 3 + k]) * s;
        q[j] = (R[j * 3 + i] + R[i * 3 + j]) * s;
        q[k] = (R[k * 3 + i] + R[i * 3 + k]) * s;
    }
}

NAVBA_HD void rot_from_q(const double* q, double* R) {
    const double tx = 2 * q[0], ty = 2 * q[1], tz = 2 * q[2];
    const double twx = tx * q[3], twy = ty * q[3], twz = tz * q[3];
    const double txx = tx * q[0], txy = ty * q[0], txz = tz * q[0];
    const double tyy = ty * q[1], tyz = tz * q[1], tzz = tz * q[2];
    R[0] = 1 - (tyy + tzz); R[1] = txy - twz;       R[2] = txz + twy;
    R[3] = txy + twz;       R[4] = 1 - (txx + tzz); R[5] = tyz - twx;
    R[6] = txz - twy;       R[7] = tyz + twx;       R[8] = 1 - (txx + tyy);
}

NAVBA_HD void q_rotate(const double* q, const double* v, double* o) {
    double uv0 = q[1] * v[2] - q[2] * v[1], uv1 = q[2] * v[0] - q[0] * v[2], uv2 = q[0] * v[1] - q[1] * v[0];
    uv0 += uv0; uv1 += uv1; uv2 += uv2;
    o[0] = v[0] + q[3] * uv0 + (q[1] * uv2 - q[2] * uv1);
    o[1] = v[1] + q[3] * uv1 + (q[2] * uv0 - q[0] * uv2);
    o[2] = v[2] + q[3] * uv2 + (q[0] * uv1 - q[1] * uv0);
}

NAVBA_HD void q_mul(const double* a, const double* b, double* r) {
    r[3] = a[3] * b[3] - a[0] * b[0] - a[1] * b[1] - a[2] * b[2];
    r[0] = a[3] * b[0] + a[0] * b[3] + a[1] * b[2] - a[2] * b[1];
    r[1] = a[3] * b[1] + a[1] * b[3] + a[2] * b[0] - a[0] * b[2];
    r[2] = a[3] * b[2] + a[2] * b[3] + a[0] * b[1] - a[1] * b[0];
}

// Pose state of one camera: q (4), t (3), pad, R (9) derived from q, pad -> 18 doubles.
struct CamState {
    double q[4];
    double t[3];
    double pad0;
    double R[9];
    double pad1;
};

// The complement of EdgeSE3ProjectXYZ::isDepthPositive (core/dataTypes/optimization/
// OptimizableTypes.hpp:109-113): the point X lies at or behind the camera, Z_c <= 0 (FP64).
NAVBA_HD bool depth_nonpositive(const CamState& c, const double* X) {
    return c.R[6] * X[0] + c.R[7] * X[1] + c.R[8] * X[2] + c.t[2] <= 0.0;
}

NAVBA_HD void cam_from_pose12(const double* P, CamState& c) {
    const double R[9] = {P[0], P[1], P[2], P[4], P[5], P[6], P[8], P[9], P[10]};
    q_from_rot(R, c.q);
    q_normalize(c.q);
    c.t[0] = P[3]; c.t[1] = P[7]; c.t[2] = P[11];
    rot_from_q(c.q, c.R);
    c.pad0 = 0.0;
    c.pad1 = 0.0;
}

NAVBA_HD void pose12_from_cam(const CamState& c, double* P) {
    for (int r = 0; r < 3; ++r) {
        P[r * 4 + 0] = c.R[r * 3 + 0];
        P[r * 4 + 1] = c.R[r * 3 + 1];
        P[r * 4 + 2] = c.R[r * 3 + 2];
        P[r * 4 + 3] = c.t[r];
    }
}

// T <- exp(d) * T with g2o's SE3Quat::exp (small-angle branch R = V = I + W + W^2 for
// |omega| < 1e-5) and SE3Quat::operator* (t = t_d + q_d t, q = q_d q, normalized).
NAVBA_HD void se3_left_update(const double* d, const CamState& in, CamState& out) {
    const double w0 = d[0], w1 = d[1], w2 = d[2];
    const double th = sqrt(w0 * w0 + w1 * w1 + w2 * w2);
    const double W[9] = {0, -w2, w1, w2, 0, -w0, -w1, w0, 0};
    double W2[9];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            W2[i * 3 + j] = W[i * 3 + 0] * W[0 * 3 + j] + W[i * 3 + 1] * W[1 * 3 + j] + W[i * 3 + 2] * W[2 * 3 + j];
    double R[9], V[9];
    if (th < 0.00001) {
        for (int k = 0; k < 9; ++k) R[k] = ((k % 4) == 0 ? 1.0 : 0.0) + W[k] + W2[k];
        for (int k = 0; k < 9; ++k) V[k] = R[k];
    } else {
        double s, c;
        sincos(th, &s, &c);
        const double a = s / th;
        const double b = (1 - c) / (th * th);
        const double cc = (th - s) / (th * th * th);
        for (int k = 0; k < 9; ++k) R[k] = ((k % 4) == 0 ? 1.0 : 0.0) + a * W[k] + b * W2[k];
        for (int k = 0; k < 9; ++k) V[k] = ((k % 4) == 0 ? 1.0 : 0.0) + b * W[k] + cc * W2[k];
    }
    double qd[4];
    q_from_rot(R, qd);
    q_normalize(qd);
    double td[3];
    for (int i = 0; i < 3; ++i) td[i] = V[i * 3 + 0] * d[3] + V[i * 3 + 1] * d[4] + V[i * 3 + 2] * d[5];
    double rt[3];
    q_rotate(qd, in.t, rt);
    for (int i = 0; i < 3; ++i) out.t[i] = td[i] + rt[i];
    q_mul(qd, in.q, out.q);
    q_normalize(out.q);
    rot_from_q(out.q, out.R);
    out.pad0 = 0.0;
    out.pad1 = 0.0;
}

// The step exp(d) of se3_left_update as E - I (row-major 3x3) and E_t = V upsilon, with the same
// branches, without forming I + (small term): the change of a transformed point under the step,
// (E - I) y + E_t, keeps its relative precision when rounded to FP32.
NAVBA_HD void se3_exp_delta(const double* d, double* EmI, double* Et) {
    const double w0 = d[0], w1 = d[1], w2 = d[2];
    const double th = sqrt(w0 * w0 + w1 * w1 + w2 * w2);
    const double W[9] = {0, -w2, w1, w2, 0, -w0, -w1, w0, 0};
    double W2[9];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            W2[i * 3 + j] = W[i * 3 + 0] * W[0 * 3 + j] + W[i * 3 + 1] * W[1 * 3 + j] + W[i * 3 + 2] * W[2 * 3 + j];
    double a = 1.0, b = 1.0, cc = 1.0, vb = 1.0;  // small-angle branch: R = V = I + W + W^2
    if (!(th < 0.00001)) {
        double s, c;
        sincos(th, &s, &c);
        a = s / th;
        b = (1 - c) / (th * th);
        cc = (th - s) / (th * th * th);
        vb = b;
    }
    for (int k = 0; k < 9; ++k) EmI[k] = a * W[k] + b * W2[k];
    // V - I = vb W + cc W^2 (small-angle: W + W^2)
    for (int i = 0; i < 3; ++i) {
        double v = d[3 + i];
        for (int j = 0; j < 3; ++j) v += (vb * W[i * 3 + j] + cc * W2[i * 3 + j]) * d[3 + j];
        Et[i] = v;
    }
}

// ---- edge ------------------------------------------------------------------------------

template <class Real>
struct EdgeLin {
    Real e[2];
    Real jc[12];  // 2x6, rotation first
    Real jp[6];   // 2x3
    Real jk[4];   // 2x2 d e / d (k1, k2) (radial model; zero for the pinhole)
    Real w;       // rho'(e^T e)
    double rho;   // rho(e^T e)
    Real xc[3];   // the point in the camera
};

// Huber (g2o RobustKernelHuber::robustify): rho(s) = s for s <= d^2 else 2 d sqrt(s) - d^2,
// rho'(s) = 1 or d / sqrt(s).
template <class Real>
NAVBA_HD void huber(Real s, bool robust, Real delta, double& rho, Real& w) {
    if (!robust || s <= delta * delta) {
        rho = (double)s;
        w = Real(1);
    } else {
        const Real r = sqrt(s);
        rho = (double)(Real(2) * r * delta - delta * delta);
        w = delta / r;
    }
}

// Camera-frame point Xc = R X + t in precision Real.
template <class Real>
NAVBA_HD void transform(const Real* R, const Real* t, const Real* X, Real* Xc) {
    Xc[0] = R[0] * X[0] + R[1] * X[1] + R[2] * X[2] + t[0];
    Xc[1] = R[3] * X[0] + R[4] * X[1] + R[5] * X[2] + t[1];
    Xc[2] = R[6] * X[0] + R[7] * X[1] + R[8] * X[2] + t[2];
}

// 1/z.  In FP64 on the device by Newton-Raphson for the reciprocal (x <- x + x (1 - z x), quadratic
// convergence) from the FP32 reciprocal: its ~2^-23 relative error falls below an ulp in two steps
// (at most 1 ulp from the IEEE quotient: tests/test_gpu_nr_math.py over 1e-20..1e20).  The IEEE
// FP64 divide is a long instruction sequence on GB300's FP64 pipe; this is two conversions and four
// fused multiply-adds.  Outside the FP32 range, and in FP32 or on the host, the plain quotient.
template <class Real>
NAVBA_HD Real recip(Real z) {
#ifdef __CUDA_ARCH__
    if constexpr (sizeof(Real) == 8) {
        const double az = fabs(z);
        if (az > 1e-30 && az < 1e30) {
            double x = (double)(1.0f / (float)z);
            x = fma(x, fma(-z, x, 1.0), x);
            x = fma(x, fma(-z, x, 1.0), x);
            return x;
        }
    }
#endif
    return Real(1) / z;
}

#ifdef __CUDACC__
// FP64 reciprocal and reciprocal square root by Newton-Raphson from the FP32 estimate (device):
// x <- x (2 - z x) and r <- r (3 - y r^2) / 2 converge quadratically, so the estimate's ~2^-22
// relative error falls to the FP64 rounding level in two steps.  Outside the FP32 range the IEEE
// operations are used.  Bounded against the IEEE results in ulps by tests/test_gpu_nr_math.py.
__device__ __forceinline__ double recip_nr(double z) { return recip<double>(z); }

__device__ __forceinline__ double rsqrt_nr(double y) {
    if (y > 1e-30 && y < 1e30) {
        double r = (double)rsqrtf((float)y);
        r = r * fma(-0.5 * y * r, r, 1.5);
        r = r * fma(-0.5 * y * r, r, 1.5);
        return r;
    }
    return 1.0 / sqrt(y);
}
#endif

// Projection pi(Xc) and, if J != nullptr, d pi / d Xc (2x3); if Jk != nullptr (radial model),
// d pi / d (k1, k2) (2x2).
template <class Real>
NAVBA_HD void project(const Intr& in, const Real* Xc, Real* uv, Real* J, Real* Jk = nullptr) {
    const Real x = Xc[0], y = Xc[1], z = Xc[2];
    const IntrV<Real> kv = intr_in<Real>(in);
    const Real fx = kv.fx, fy = kv.fy, cx = kv.cx, cy = kv.cy;
    if (in.model == 2) {
        // Kannala-Brandt (KannalaBrandt8.cpp:80-107 projection, :195-226 Jacobian), in Real throughout:
        // pi = f r(theta) (x, y) / rho + c, theta = atan2(rho, z), r = theta + k1 theta^3 + .. + k4 theta^9.
        // (The reference rounds theta and psi to float in project; here they keep Real precision.)
        // With A = r'(theta) z / (rho^2 + z^2) and B = r / rho the Jacobian is
        //   [[fx (x^2 A + y^2 B), fx x y (A - B)] / rho^2, -fx r' x / (rho^2 + z^2)], likewise for v;
        // on the optical axis (rho <= 1e-9 |z|) both reduce to the pinhole values (B -> 1/z).
        const Real k1 = kv.k1, k2 = kv.k2, k3 = kv.k3, k4 = kv.k4;
        const Real rho2 = x * x + y * y, rho = sqrt(rho2);
        const Real rz2 = rho2 + z * z;
        if (rho <= Real(1e-9) * fabs(z)) {
            const Real iz = Real(1) / z;
            uv[0] = fx * x * iz + cx;
            uv[1] = fy * y * iz + cy;
            if (J) {
                J[0] = fx * iz; J[1] = Real(0); J[2] = -fx * x * iz * iz;
                J[3] = Real(0); J[4] = fy * iz; J[5] = -fy * y * iz * iz;
            }
        } else {
            const Real th = atan2(rho, z), t2 = th * th;
            const Real r = th * (Real(1) + t2 * (k1 + t2 * (k2 + t2 * (k3 + t2 * k4))));
            const Real B = r / rho;
            uv[0] = fx * B * x + cx;
            uv[1] = fy * B * y + cy;
            if (J) {
                const Real rd = Real(1) + t2 * (Real(3) * k1 + t2 * (Real(5) * k2 + t2 * (Real(7) * k3 + t2 * Real(9) * k4)));
                const Real A = rd * z / rz2;
                const Real ir2 = Real(1) / rho2;
                J[0] = fx * (x * x * A + y * y * B) * ir2;
                J[1] = fx * x * y * (A - B) * ir2;
                J[2] = -fx * rd * x / rz2;
                J[3] = fy * x * y * (A - B) * ir2;
                J[4] = fy * (y * y * A + x * x * B) * ir2;
                J[5] = -fy * rd * y / rz2;
            }
        }
        return;
    }
    const Real iz = recip(z);  // one reciprocal per edge; the rest are products
    if (in.model == 0) {
        const Real xn = x * iz, yn = y * iz;
        uv[0] = fx * xn + cx;
        uv[1] = fy * yn + cy;
        if (J) {
            J[0] = fx * iz; J[1] = Real(0); J[2] = -fx * xn * iz;
            J[3] = Real(0); J[4] = fy * iz; J[5] = -fy * yn * iz;
        }
    } else {
        const Real k1 = kv.k1, k2 = kv.k2;
        const Real xn = x * iz, yn = y * iz;
        const Real r2 = xn * xn + yn * yn;
        const Real d = Real(1) + k1 * r2 + k2 * r2 * r2;
        uv[0] = fx * d * xn + cx;
        uv[1] = fy * d * yn + cy;
        if (J) {
            const Real c = k1 + Real(2) * k2 * r2;
            const Real a00 = fx * (d + Real(2) * xn * xn * c), a01 = fx * Real(2) * xn * yn * c;
            const Real a10 = fy * Real(2) * xn * yn * c, a11 = fy * (d + Real(2) * yn * yn * c);
            J[0] = a00 * iz; J[1] = a01 * iz; J[2] = -(a00 * xn + a01 * yn) * iz;
            J[3] = a10 * iz; J[4] = a11 * iz; J[5] = -(a10 * xn + a11 * yn) * iz;
        }
        if (Jk) {
            Jk[0] = fx * xn * r2; Jk[1] = fx * xn * r2 * r2;
            Jk[2] = fy * yn * r2; Jk[3] = fy * yn * r2 * r2;
        }
    }
}

// Residual, Jacobians and robust weight of one edge (EdgeSE3ProjectXYZ::computeError and
// ::linearizeOplus).  R, t: camera rotation/translation; X: world point; z: measurement.
template <class Real>
NAVBA_HD void edge_linearize(const Intr& in, const Real* R, const Real* t, const Real* X,
                             const Real* z, bool robust, Real delta, EdgeLin<Real>& L) {
    Real Xc[3], uv[2], J[6], Jk[4] = {Real(0), Real(0), Real(0), Real(0)};
    transform(R, t, X, Xc);
    L.xc[0] = Xc[0];
    L.xc[1] = Xc[1];
    L.xc[2] = Xc[2];
    project(in, Xc, uv, J, in.model == 1 ? Jk : nullptr);
    L.e[0] = z[0] - uv[0];
    L.e[1] = z[1] - uv[1];
    L.jk[0] = -Jk[0]; L.jk[1] = -Jk[1]; L.jk[2] = -Jk[2]; L.jk[3] = -Jk[3];
    huber<Real>(L.e[0] * L.e[0] + L.e[1] * L.e[1], robust, delta, L.rho, L.w);
    Real P[6];
    for (int k = 0; k < 6; ++k) P[k] = -J[k];
#pragma unroll
    for (int r = 0; r < 2; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c)
            L.jp[r * 3 + c] = P[r * 3 + 0] * R[0 * 3 + c] + P[r * 3 + 1] * R[1 * 3 + c] + P[r * 3 + 2] * R[2 * 3 + c];
    const Real x = Xc[0], y = Xc[1], zc = Xc[2];
    // J_pose = P * [[0, z, -y, 1, 0, 0], [-z, 0, x, 0, 1, 0], [y, -x, 0, 0, 0, 1]]
#pragma unroll
    for (int r = 0; r < 2; ++r) {
        const Real p0 = P[r * 3 + 0], p1 = P[r * 3 + 1], p2 = P[r * 3 + 2];
        L.jc[r * 6 + 0] = -p1 * zc + p2 * y;
        L.jc[r * 6 + 1] = p0 * zc - p2 * x;
        L.jc[r * 6 + 2] = -p0 * y + p1 * x;
        L.jc[r * 6 + 3] = p0;
        L.jc[r * 6 + 4] = p1;
        L.jc[r * 6 + 5] = p2;
    }
}

// Pinhole pose Jacobian d e / d (omega, upsilon) (edge_linearize's jc, rotation first) from the
// normalized camera coordinates u = x / z, v = y / z and iz = 1 / z of the point in the camera:
// -Jpi [-[Xc]x | I] with Jpi = iz [[fx, 0, -fx u], [0, fy, -fy v]]; the rotation block does not
// depend on the depth.
template <class Real>
NAVBA_HD void pinhole_jc(Real fx, Real fy, Real u, Real v, Real iz, Real* jc) {
    const Real uv = u * v;
    jc[0] = fx * uv;
    jc[1] = -fx * (Real(1) + u * u);
    jc[2] = fx * v;
    jc[3] = -fx * iz;
    jc[4] = Real(0);
    jc[5] = fx * u * iz;
    jc[6] = fy * (Real(1) + v * v);
    jc[7] = -fy * uv;
    jc[8] = -fy * u;
    jc[9] = Real(0);
    jc[10] = -fy * iz;
    jc[11] = fy * v * iz;
}

// Robust chi2 of one edge, in precision Real.
template <class Real>
NAVBA_HD double edge_cost(const Intr& in, const Real* R, const Real* t, const Real* X,
                          const Real* z, bool robust, Real delta) {
    Real Xc[3], uv[2];
    transform(R, t, X, Xc);
    project<Real>(in, Xc, uv, nullptr);
    const Real e0 = z[0] - uv[0], e1 = z[1] - uv[1];
    double rho;
    Real w;
    huber<Real>(e0 * e0 + e1 * e1, robust, delta, rho, w);
    return rho;
}

// Inverse of a symmetric 3x3 (packed a00 a01 a02 a11 a12 a22) by its adjugate; returns the
// packed inverse.  Same formula as Eigen's fixed-size inverse used by g2o's Schur step.
template <class Real>
NAVBA_HD void inv_sym3(const Real* v, Real* o) {
    const Real m00 = v[0], m01 = v[1], m02 = v[2], m11 = v[3], m12 = v[4], m22 = v[5];
    const Real c00 = m11 * m22 - m12 * m12;
    const Real c10 = m12 * m02 - m01 * m22;
    const Real c20 = m01 * m12 - m11 * m02;
    const Real det = m00 * c00 + m01 * c10 + m02 * c20;
    const Real id = Real(1) / det;
    o[0] = c00 * id;
    o[1] = (m02 * m12 - m01 * m22) * id;
    o[2] = (m01 * m12 - m02 * m11) * id;
    o[3] = (m00 * m22 - m02 * m02) * id;
    o[4] = (m02 * m01 - m00 * m12) * id;
    o[5] = (m00 * m11 - m01 * m01) * id;
}

}  // namespace navba
