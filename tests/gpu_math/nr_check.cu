// nr_check.cu - test harness (built by tests/test_gpu_nr_math.py): evaluates the library's FP64
// Newton-Raphson reciprocal and reciprocal square root (nav24_gb300/csrc/ba_math.cuh) on the device
// next to the IEEE operations, for the ulp bounds the test asserts.
#include <cuda_runtime.h>

#include "../../nav24_gb300/csrc/ba_math.cuh"

namespace {

// out[i] = {recip_nr(z), 1/z, rsqrt_nr(|z|), 1/sqrt(|z|)} for each input z[i].
__global__ void k_nr(const double* z, int n, double* out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double v = z[i], a = fabs(v);
    out[4LL * i + 0] = navba::recip_nr(v);
    out[4LL * i + 1] = 1.0 / v;
    out[4LL * i + 2] = navba::rsqrt_nr(a);
    out[4LL * i + 3] = 1.0 / sqrt(a);
}

}  // namespace

extern "C" int nr_eval(const double* z, int n, double* out) {
    double *dz = nullptr, *dout = nullptr;
    cudaError_t e = cudaMalloc(&dz, sizeof(double) * (size_t)n);
    if (e == cudaSuccess) e = cudaMalloc(&dout, sizeof(double) * 4 * (size_t)n);
    if (e == cudaSuccess) e = cudaMemcpy(dz, z, sizeof(double) * (size_t)n, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        k_nr<<<(n + 255) / 256, 256>>>(dz, n, dout);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(out, dout, sizeof(double) * 4 * (size_t)n, cudaMemcpyDeviceToHost);
    cudaFree(dz);
    cudaFree(dout);
    return (int)e;
}
