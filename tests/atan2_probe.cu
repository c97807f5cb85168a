// Test helper (built by tests/test_atan2_gpu.py): evaluates the engine's
// arctangent polynomials (atan2_poly, atan2_bins and their f32x2 pair forms
// atan2_poly2 and atan2_bins2, element i paired with element i ^ 1) and
// CUDA's atan2f on the device for the same inputs.
#include <cuda_runtime.h>

#include "../sift_wgpu_gb300/csrc/sift_internal.cuh"

namespace {
__global__ void k_atan2_probe(const float* __restrict__ y, const float* __restrict__ x, int n, float* __restrict__ poly,
                              float* __restrict__ bins, float* __restrict__ bins2, float* __restrict__ poly2,
                              float* __restrict__ ref) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    poly[i] = sift::atan2_poly(y[i], x[i]);
    bins[i] = sift::atan2_bins(y[i], x[i]);
    const int j = (i ^ 1) < n ? (i ^ 1) : i;
    const float2 b2 = sift::atan2_bins2(make_float2(y[i], y[j]), make_float2(x[i], x[j]));
    bins2[i] = b2.x;
    poly2[i] = sift::atan2_poly2(make_float2(y[i], y[j]), make_float2(x[i], x[j])).x;
    ref[i] = atan2f(y[i], x[i]);
}
}  // namespace

extern "C" int atan2_probe(const float* hy, const float* hx, int n, float* hpoly, float* hbins, float* hbins2,
                           float* hpoly2, float* href) {
    if (n <= 0) return 0;
    float* d = nullptr;
    const size_t b = (size_t)n * sizeof(float);
    if (cudaMalloc(&d, 7 * b) != cudaSuccess) return 1;
    float *dy = d, *dx = d + n, *dp = d + 2 * (size_t)n, *db = d + 3 * (size_t)n, *dr = d + 4 * (size_t)n;
    float* db2 = d + 5 * (size_t)n;
    float* dp2 = d + 6 * (size_t)n;
    int rc = 0;
    if (cudaMemcpy(dy, hy, b, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(dx, hx, b, cudaMemcpyHostToDevice) != cudaSuccess)
        rc = 2;
    if (!rc) {
        k_atan2_probe<<<(n + 255) / 256, 256>>>(dy, dx, n, dp, db, db2, dp2, dr);
        if (cudaGetLastError() != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess) rc = 3;
    }
    if (!rc && (cudaMemcpy(hpoly, dp, b, cudaMemcpyDeviceToHost) != cudaSuccess ||
                cudaMemcpy(hbins, db, b, cudaMemcpyDeviceToHost) != cudaSuccess ||
                cudaMemcpy(hbins2, db2, b, cudaMemcpyDeviceToHost) != cudaSuccess ||
                cudaMemcpy(hpoly2, dp2, b, cudaMemcpyDeviceToHost) != cudaSuccess ||
                cudaMemcpy(href, dr, b, cudaMemcpyDeviceToHost) != cudaSuccess))
        rc = 4;
    cudaFree(d);
    return rc;
}
