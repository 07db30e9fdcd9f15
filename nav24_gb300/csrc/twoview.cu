// twoview.cu - two-view triangulation and the per-match checks of map initialization, for every
// (relative-pose hypothesis, match) pair in one launch (thread per pair).
//
// TwoViewReconstruction::Triangulate (core/operators/mapInit/OP_2ViewReconstruction.cpp:1179-1193)
// takes the right singular vector of the 4x4 DLT matrix A for its smallest singular value; here it
// comes from a one-sided Jacobi SVD of the same A, in FP64 (the reference: cv::SVD on CV_32F).
// The per-match host work (nGood, the k-th smallest parallax cosine) is linear in the matches.
// The checks follow TwoViewReconstruction::CheckRT (:1244-1353) in order.  The reductions CheckRT
// makes over matches (nGood, the parallax statistic) are formed on the host from the flags.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "engine.hpp"

namespace navba {
namespace {

struct TvArgs {
    int n, nh;
    double fx, fy, cx, cy;
    const double* kp1;
    const double* kp2;
    const uint8_t* inl;
    const double* R;
    const double* t;
    double th2, minpc;
    double* pts;     // [nh][n][3]
    uint8_t* flags;  // [nh][n]: 1 triangulated, 2 good
    double* cosp;    // [nh][n]
};

// The rotation parameters' FP64 reciprocals and reciprocal square roots are Newton-Raphson
// refinements of FP32 estimates (recip_nr, rsqrt_nr in ba_math.cuh): GB300 issues FP64 at 2 lanes
// per clock per SM, the IEEE divide and square root are long sequences, and the rotations are this
// kernel's FP64 work.

// Right singular vector of a 4x4 matrix for its smallest singular value: one-sided Jacobi
// (Hestenes 1958): column pairs of A are rotated until mutually orthogonal, the rotations
// accumulate in V, and the column of V belonging to the shortest column of A is the vector.
// At most 20 sweeps over the 6 column pairs.
__device__ void svd4_min_right(double A[4][4], double v[4]) {
    double V[4][4] = {{1, 0, 0, 0}, {0, 1, 0, 0}, {0, 0, 1, 0}, {0, 0, 0, 1}};
    for (int sweep = 0; sweep < 20; ++sweep) {
        bool rotated = false;
        for (int p = 0; p < 3; ++p)
            for (int q = p + 1; q < 4; ++q) {
                double al = 0.0, be = 0.0, ga = 0.0;
                for (int k = 0; k < 4; ++k) {
                    al += A[k][p] * A[k][p];
                    be += A[k][q] * A[k][q];
                    ga += A[k][p] * A[k][q];
                }
                if (!(ga * ga > 1e-30 * (al * be))) continue;  // |ga| > 1e-15 sqrt(al be)
                rotated = true;
                // tan of the rotation angle: sign(ze) / (|ze| + sqrt(1 + ze^2)), or 1 / (2 ze) once
                // sqrt(1 + ze^2) = |ze| in FP64
                const double ze = (be - al) * recip_nr(2.0 * ga);
                const double aze = fabs(ze);
                double tt;
                if (aze < 1e15) {
                    const double y = 1.0 + ze * ze;
                    tt = (ze >= 0 ? 1.0 : -1.0) * recip_nr(aze + y * rsqrt_nr(y));
                } else {
                    tt = 0.5 * recip_nr(ze);
                }
                const double c = rsqrt_nr(1.0 + tt * tt), s = c * tt;
                for (int k = 0; k < 4; ++k) {
                    const double a = A[k][p], b = A[k][q];
                    A[k][p] = c * a - s * b;
                    A[k][q] = s * a + c * b;
                    const double va = V[k][p], vb = V[k][q];
                    V[k][p] = c * va - s * vb;
                    V[k][q] = s * va + c * vb;
                }
            }
        if (!rotated) break;
    }
    int im = 0;
    double nm = 1e300;
    for (int j = 0; j < 4; ++j) {
        const double nj = A[0][j] * A[0][j] + A[1][j] * A[1][j] + A[2][j] * A[2][j] + A[3][j] * A[3][j];
        if (nj < nm) {
            nm = nj;
            im = j;
        }
    }
    for (int k = 0; k < 4; ++k) v[k] = V[k][im];
}

__global__ void k_twoview(TvArgs A) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)A.n * A.nh) return;
    const int h = (int)(idx / A.n), i = (int)(idx % A.n);
    double* X = A.pts + 3 * idx;
    X[0] = X[1] = X[2] = nan("");
    A.flags[idx] = 0;
    A.cosp[idx] = nan("");
    if (A.inl && !A.inl[i]) return;
    const double* R = A.R + 9LL * h;
    const double* t = A.t + 3LL * h;
    const double x1 = A.kp1[2LL * i], y1 = A.kp1[2LL * i + 1], x2 = A.kp2[2LL * i], y2 = A.kp2[2LL * i + 1];
    // P1 = K [I | 0], P2 = K [R | t]
    const double P1[3][4] = {{A.fx, 0, A.cx, 0}, {0, A.fy, A.cy, 0}, {0, 0, 1, 0}};
    double P2[3][4];
    for (int c = 0; c < 4; ++c) {
        const double r0 = c < 3 ? R[c] : t[0], r1 = c < 3 ? R[3 + c] : t[1], r2 = c < 3 ? R[6 + c] : t[2];
        P2[0][c] = A.fx * r0 + A.cx * r2;
        P2[1][c] = A.fy * r1 + A.cy * r2;
        P2[2][c] = r2;
    }
    double Am[4][4];
    for (int c = 0; c < 4; ++c) {
        Am[0][c] = x1 * P1[2][c] - P1[0][c];
        Am[1][c] = y1 * P1[2][c] - P1[1][c];
        Am[2][c] = x2 * P2[2][c] - P2[0][c];
        Am[3][c] = y2 * P2[2][c] - P2[1][c];
    }
    double v[4];
    svd4_min_right(Am, v);
    const double p[3] = {v[0] / v[3], v[1] / v[3], v[2] / v[3]};
    if (!isfinite(p[0]) || !isfinite(p[1]) || !isfinite(p[2])) return;
    X[0] = p[0];
    X[1] = p[1];
    X[2] = p[2];
    // parallax between the rays from O1 = 0 and O2 = -R^T t
    const double O2[3] = {-(R[0] * t[0] + R[3] * t[1] + R[6] * t[2]), -(R[1] * t[0] + R[4] * t[1] + R[7] * t[2]),
                          -(R[2] * t[0] + R[5] * t[1] + R[8] * t[2])};
    const double n2[3] = {p[0] - O2[0], p[1] - O2[1], p[2] - O2[2]};
    const double d1 = sqrt(p[0] * p[0] + p[1] * p[1] + p[2] * p[2]);
    const double d2 = sqrt(n2[0] * n2[0] + n2[1] * n2[1] + n2[2] * n2[2]);
    const double cp = (p[0] * n2[0] + p[1] * n2[1] + p[2] * n2[2]) / (d1 * d2);
    A.cosp[idx] = cp;
    if (p[2] <= 0 && cp < A.minpc) return;
    const double q[3] = {R[0] * p[0] + R[1] * p[1] + R[2] * p[2] + t[0], R[3] * p[0] + R[4] * p[1] + R[5] * p[2] + t[1],
                         R[6] * p[0] + R[7] * p[1] + R[8] * p[2] + t[2]};
    if (q[2] <= 0 && cp < A.minpc) return;
    const double u1 = A.fx * p[0] / p[2] + A.cx - x1, w1 = A.fy * p[1] / p[2] + A.cy - y1;
    if (u1 * u1 + w1 * w1 > A.th2) return;
    const double u2 = A.fx * q[0] / q[2] + A.cx - x2, w2 = A.fy * q[1] / q[2] + A.cy - y2;
    if (u2 * u2 + w2 * w2 > A.th2) return;
    A.flags[idx] = (uint8_t)(1 | (cp < A.minpc ? 2 : 0));
}

bool all_finite(const double* p, int64_t n) {
    for (int64_t i = 0; i < n; ++i)
        if (!std::isfinite(p[i])) return false;
    return true;
}

}  // namespace

nav_ba_status twoview_check(cudaStream_t st, const nav_ba_twoview& in, nav_ba_twoview_result& out, std::string* why,
                            DevScratch& scratch) {
    const int n = in.n_matches, nh = in.n_hyp;
    if (n < 0 || nh < 0 || (n > 0 && (!in.kp1 || !in.kp2)) || (nh > 0 && (!in.R || !in.t)) ||
        (nh > 0 && (!out.n_good || !out.parallax_deg))) {
        *why = "NULL array or negative size";
        return NAV_BA_ERR_ARGUMENT;
    }
    if (!all_finite(in.K, 4) || !all_finite(in.kp1, 2LL * n) || !all_finite(in.kp2, 2LL * n) ||
        !all_finite(in.R, 9LL * nh) || !all_finite(in.t, 3LL * nh) || !std::isfinite(in.th2) ||
        !std::isfinite(in.min_parallax_cos)) {
        *why = "non-finite input";
        return NAV_BA_ERR_NONFINITE_INPUT;
    }
    const int64_t m = (int64_t)n * nh;
    // host copies of the per-pair outputs (default-initialized: every entry is read back); the
    // points go straight to the caller's buffer when it gives one
    std::unique_ptr<double[]> pts_own(out.points ? nullptr : new double[3 * std::max<int64_t>(m, 1)]);
    double* pts = out.points ? out.points : pts_own.get();
    std::unique_ptr<double[]> cosp(new double[std::max<int64_t>(m, 1)]);
    std::unique_ptr<uint8_t[]> flags(new uint8_t[std::max<int64_t>(m, 1)]);
    if (m > 0) {
        const size_t b_kp = sizeof(double) * 2 * n, b_in = in.inlier ? (size_t)n : 0, b_R = sizeof(double) * 9 * nh,
                     b_t = sizeof(double) * 3 * nh, b_pts = sizeof(double) * 3 * m, b_cos = sizeof(double) * m,
                     b_fl = (size_t)m;
        auto up16 = [](size_t x) { return (x + 255) & ~(size_t)255; };
        const size_t o_kp1 = 0, o_kp2 = o_kp1 + up16(b_kp), o_in = o_kp2 + up16(b_kp), o_R = o_in + up16(b_in),
                     o_t = o_R + up16(b_R), o_pts = o_t + up16(b_t), o_cos = o_pts + up16(b_pts), o_fl = o_cos + up16(b_cos),
                     total = o_fl + up16(b_fl);
        cudaError_t e = cudaSuccess;
        auto* base = static_cast<unsigned char*>(scratch.get(total, &e));
        auto upl = [&](size_t off, const void* h, size_t bytes) {
            if (e == cudaSuccess && bytes) e = cudaMemcpyAsync(base + off, h, bytes, cudaMemcpyHostToDevice, st);
        };
        upl(o_kp1, in.kp1, b_kp);
        upl(o_kp2, in.kp2, b_kp);
        upl(o_in, in.inlier, b_in);
        upl(o_R, in.R, b_R);
        upl(o_t, in.t, b_t);
        TvArgs A;
        A.n = n;
        A.nh = nh;
        A.fx = in.K[0];
        A.fy = in.K[1];
        A.cx = in.K[2];
        A.cy = in.K[3];
        A.kp1 = reinterpret_cast<const double*>(base + o_kp1);
        A.kp2 = reinterpret_cast<const double*>(base + o_kp2);
        A.inl = in.inlier ? base + o_in : nullptr;
        A.R = reinterpret_cast<const double*>(base + o_R);
        A.t = reinterpret_cast<const double*>(base + o_t);
        A.th2 = in.th2;
        A.minpc = in.min_parallax_cos;
        A.pts = reinterpret_cast<double*>(base + o_pts);
        A.cosp = reinterpret_cast<double*>(base + o_cos);
        A.flags = base + o_fl;
        if (e == cudaSuccess) {
            k_twoview<<<(unsigned)((m + 127) / 128), 128, 0, st>>>(A);
            e = cudaGetLastError();
        }
        if (e == cudaSuccess) e = cudaMemcpyAsync(pts, A.pts, b_pts, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(cosp.get(), A.cosp, b_cos, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(flags.get(), A.flags, b_fl, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) {
            *why = std::string("two-view kernel: ") + cudaGetErrorString(e);
            return NAV_BA_ERR_CUDA;
        }
    }
    std::vector<double> cs;
    for (int h = 0; h < nh; ++h) {
        cs.clear();
        for (int i = 0; i < n; ++i)
            if (flags[(size_t)h * n + i] & 1) cs.push_back(cosp[(size_t)h * n + i]);
        out.n_good[h] = (int32_t)cs.size();
        if (cs.empty()) {
            out.parallax_deg[h] = 0.0;
        } else {
            // the k-th smallest cosine, the element CheckRT reads after sorting them all
            const size_t k = std::min<size_t>((size_t)std::max(0, in.min_triangulated), cs.size() - 1);
            std::nth_element(cs.begin(), cs.begin() + k, cs.end());
            out.parallax_deg[h] = std::acos(cs[k]) * 180.0 / M_PI;
        }
    }
    for (int64_t k = 0; k < m; ++k) {
        if (out.triangulated) out.triangulated[k] = flags[k] & 1;
        if (out.good) out.good[k] = (flags[k] >> 1) & 1;
    }
    return NAV_BA_OK;
}

}  // namespace navba
