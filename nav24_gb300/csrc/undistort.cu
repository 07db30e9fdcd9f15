// undistort.cu - keypoint undistortion for the radial-tangential pinhole, thread per keypoint.
//
// nav24 undistorts every keypoint before BA (Calibration::undistort, core/sensor/camera/
// Calibration.cpp:135-148 -> PinholeRadTan::UndistortKeyPoints, core/sensor/camera/models/
// PinholeRadTan.cpp:11-24 -> cv::undistortPoints with R = I and P = K, distortion (k1, k2, p1, p2)).
// OpenCV (>= 4.2.0, core/CMakeLists.txt:10) inverts the distortion by a fixed-point iteration on
// normalized coordinates, x <- (x_d - dx(x)) / (1 + k1 r^2 + k2 r^4) with the tangential terms
// dx = 2 p1 x y + p2 (r^2 + 2 x^2), dy = p1 (r^2 + 2 y^2) + 2 p2 x y, a fixed number of times (its
// default criteria: 5 iterations); the result is mapped back through K.  FP64 here.
#include <cmath>
#include <string>

#include "engine.hpp"

namespace navba {
namespace {

__global__ void k_undistort(int n, double fx, double fy, double cx, double cy, double k1, double k2, double p1,
                            double p2, int iters, const double2* in, double2* out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double2 uv = in[i];
    const double x0 = (uv.x - cx) / fx, y0 = (uv.y - cy) / fy;
    double x = x0, y = y0;
    for (int k = 0; k < iters; ++k) {
        const double r2 = x * x + y * y;
        const double icd = 1.0 / (1.0 + (k2 * r2 + k1) * r2);
        const double dx = 2.0 * p1 * x * y + p2 * (r2 + 2.0 * x * x);
        const double dy = p1 * (r2 + 2.0 * y * y) + 2.0 * p2 * x * y;
        x = (x0 - dx) * icd;
        y = (y0 - dy) * icd;
    }
    out[i] = make_double2(fx * x + cx, fy * y + cy);
}

}  // namespace

nav_ba_status undistort_points(cudaStream_t st, const double* K, const double* dist, int iters, int n, const double* uv_in,
                               double* uv_out, std::string* why, DevScratch& scratch) {
    if (n < 0 || !K || !dist || (n > 0 && (!uv_in || !uv_out)) || iters < 0) {
        *why = "NULL array or negative size";
        return NAV_BA_ERR_ARGUMENT;
    }
    for (int k = 0; k < 4; ++k)
        if (!std::isfinite(K[k]) || !std::isfinite(dist[k])) {
            *why = "non-finite calibration";
            return NAV_BA_ERR_NONFINITE_INPUT;
        }
    if (!(K[0] != 0.0) || !(K[1] != 0.0)) {
        *why = "zero focal length";
        return NAV_BA_ERR_ARGUMENT;
    }
    if (n == 0) return NAV_BA_OK;
    const size_t bytes = sizeof(double2) * (size_t)n;
    cudaError_t e = cudaSuccess;
    void* buf = scratch.get(2 * bytes, &e);
    double2* din = static_cast<double2*>(buf);
    double2* dout = din + n;
    if (e == cudaSuccess) e = cudaMemcpyAsync(din, uv_in, bytes, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) {
        k_undistort<<<(n + 255) / 256, 256, 0, st>>>(n, K[0], K[1], K[2], K[3], dist[0], dist[1], dist[2], dist[3], iters,
                                                     din, dout);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(uv_out, dout, bytes, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        *why = std::string("undistort kernel: ") + cudaGetErrorString(e);
        return NAV_BA_ERR_CUDA;
    }
    return NAV_BA_OK;
}

}  // namespace navba
