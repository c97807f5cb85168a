// Test helper (built by tests/test_atan2_gpu.py): evaluates the engine's two
// arctangent polynomials and CUDA's atan2f on the device for the same inputs.
#include <cuda_runtime.h>

#include "../sift_wgpu_gb300/csrc/sift_internal.cuh"

namespace {
__global__ void k_atan2_probe(const float* __restrict__ y, const float* __restrict__ x, int n, float* __restrict__ poly,
                              float* __restrict__ bins, float* __restrict__ ref) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    poly[i] = sift::atan2_poly(y[i], x[i]);
    bins[i] = sift::atan2_bins(y[i], x[i]);
    ref[i] = atan2f(y[i], x[i]);
}
}  // namespace

extern "C" int atan2_probe(const float* hy, const float* hx, int n, float* hpoly, float* hbins, float* href) {
    if (n <= 0) return 0;
    float* d = nullptr;
    const size_t b = (size_t)n * sizeof(float);
    if (cudaMalloc(&d, 5 * b) != cudaSuccess) return 1;
    float *dy = d, *dx = d + n, *dp = d + 2 * (size_t)n, *db = d + 3 * (size_t)n, *dr = d + 4 * (size_t)n;
    int rc = 0;
    if (cudaMemcpy(dy, hy, b, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(dx, hx, b, cudaMemcpyHostToDevice) != cudaSuccess)
        rc = 2;
    if (!rc) {
        k_atan2_probe<<<(n + 255) / 256, 256>>>(dy, dx, n, dp, db, dr);
        if (cudaGetLastError() != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess) rc = 3;
    }
    if (!rc && (cudaMemcpy(hpoly, dp, b, cudaMemcpyDeviceToHost) != cudaSuccess ||
                cudaMemcpy(hbins, db, b, cudaMemcpyDeviceToHost) != cudaSuccess ||
                cudaMemcpy(href, dr, b, cudaMemcpyDeviceToHost) != cudaSuccess))
        rc = 4;
    cudaFree(d);
    return rc;
}
