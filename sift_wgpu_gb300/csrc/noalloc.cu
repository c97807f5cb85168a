// noalloc.cu — a Gaussian blur of a device image that allocates nothing.
//
// sift_cuda_gaussian_blur_u8_noalloc blurs an 8-bit image already in device
// memory into a device buffer the caller owns, with the same arithmetic as
// every blur of the pyramid: imageproc 0.25.0's gaussian_blur_f32 on a u8
// image (the base blur of detect_and_compute_cpu, src/sift.rs:1200-1214, and
// the level blurs of generate_gaussian_pyramid, src/sift.rs:129-177) — taps
// (sqrt(2 pi) sigma)^-1 exp(-x^2 / (2 sigma^2)) for |x| <= ceil(2 sigma),
// clamp-to-edge, a horizontal then a vertical pass, each summed in f32 from 0
// in tap order and truncated to u8.
//
// Who needs it: a caller that must not allocate device memory on its path —
// a serving process whose memory pool has reserved the device's free memory
// up front (a cudaMalloc there fails or evicts the pool's cache), or a
// latency-bound loop where cudaFree's implicit device-wide synchronisation
// would stall the other streams. The engine entry points grow their arenas on
// demand and so cannot serve such a caller.
//
// How: the horizontal pass's u8 intermediate goes to g_blur_scratch, a fixed
// 16 MiB array compiled into this library's device code, instead of a buffer
// allocated per call. The kernels get its device address, looked up once per
// device with cudaGetSymbolAddress (the host-side name of a __device__ array
// is not a device address). The filter taps travel in the kernel parameters.
//
// Limits and rules of use
//  - width <= 8192, align16(width) * height <= 16 MiB (4096 x 4096 fits),
//    ceil(2 sigma) <= 64. Larger requests fail with SIFT_CUDA_ERR_UNSUPPORTED
//    and a message naming the limit; nothing is launched.
//  - The first call on a device looks up the scratch address, which also
//    makes the CUDA runtime load this library's device code on that device if
//    nothing has yet. Make that first call before any stream capture begins.
//  - Nothing has to start at zero: the horizontal pass writes every scratch
//    byte that the vertical pass reads, in the same call, in stream order.
//  - All calls on a device share the one scratch array. Two calls whose
//    kernels can overlap (different streams, or different host threads without
//    ordering between them) race on it and corrupt each other's output; order
//    them on one stream or synchronise between them.
//  - On success the call allocates no device or host memory; it launches two
//    kernels on `stream` and returns without synchronising.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <mutex>

#include "sift_internal.cuh"

namespace sift {

int report_error(int code, const char* msg);  // engine.cu: sets sift_cuda_last_error

namespace {

constexpr size_t kScratchBytes = size_t(16) << 20;
constexpr int kMaxWidth = 8192;
constexpr int kMaxRadius = 64;
constexpr int kTapSlots = 2 * kMaxRadius + 1 + 7;  // taps, zero padded
constexpr int kMaxDevices = 64;

static __device__ __align__(256) uint8_t g_blur_scratch[kScratchBytes];

struct BlurTaps {
    int r;
    float w[kTapSlots];
};

constexpr int kRowThreads = 128;

// Horizontal pass, one row per CTA: the clamp-to-edge row in shared memory,
// four outputs per thread, u8 results into the scratch plane.
__global__ void __launch_bounds__(kRowThreads) k_rows_to_scratch(const uint8_t* __restrict__ src,
                                                                 long long src_stride, uint8_t* __restrict__ scratch,
                                                                 int sp, int W, const __grid_constant__ BlurTaps t) {
    extern __shared__ __align__(16) float sm[];
    const int r = t.r, taps = 2 * r + 1;
    float* kw = sm;
    float* row = sm + kTapSlots + 1;
    const int y = blockIdx.x;
    const uint8_t* s = src + (long long)y * src_stride;
    for (int i = threadIdx.x; i < taps; i += blockDim.x) kw[i] = t.w[i];
    for (int j = threadIdx.x; j < W + 2 * r + 3; j += blockDim.x) row[j] = float_of_u8(s[clampi(j - r, 0, W - 1)]);
    __syncthreads();
    uint8_t* d = scratch + (long long)y * sp;
    for (int x0 = threadIdx.x * 4; x0 < W; x0 += blockDim.x * 4) {
        float a0 = 0.0f, a1 = 0.0f, a2 = 0.0f, a3 = 0.0f;
        const float* b = row + x0;
        for (int i = 0; i < taps; ++i) {
            const float k = kw[i];
            a0 = __fadd_rn(a0, __fmul_rn(b[i + 0], k));
            a1 = __fadd_rn(a1, __fmul_rn(b[i + 1], k));
            a2 = __fadd_rn(a2, __fmul_rn(b[i + 2], k));
            a3 = __fadd_rn(a3, __fmul_rn(b[i + 3], k));
        }
        d[x0] = (uint8_t)clamp_u8(a0);
        if (x0 + 1 < W) d[x0 + 1] = (uint8_t)clamp_u8(a1);
        if (x0 + 2 < W) d[x0 + 2] = (uint8_t)clamp_u8(a2);
        if (x0 + 3 < W) d[x0 + 3] = (uint8_t)clamp_u8(a3);
    }
}

constexpr int kColTX = 32, kColTY = 8, kColRPT = 8, kColRows = kColTY * kColRPT;

// Vertical pass over a 32 x 64 output tile: the scratch rows of the tile and
// its clamp-to-edge halo in shared memory, eight outputs per thread.
__global__ void __launch_bounds__(kColTX* kColTY) k_cols_from_scratch(const uint8_t* __restrict__ scratch, int sp,
                                                                     uint8_t* __restrict__ dst, long long dst_stride,
                                                                     int W, int H, const __grid_constant__ BlurTaps t) {
    extern __shared__ __align__(16) float sm[];
    const int r = t.r, taps = 2 * r + 1;
    float* kw = sm;
    float* tile = sm + kTapSlots + 1;  // [kColRows + 2r][kColTX]
    const int tid = threadIdx.y * kColTX + threadIdx.x;
    const int x0 = blockIdx.x * kColTX, y0 = blockIdx.y * kColRows;
    for (int i = tid; i < taps; i += kColTX * kColTY) kw[i] = t.w[i];
    const int xg = min(x0 + (int)threadIdx.x, W - 1);
    for (int k = threadIdx.y; k < kColRows + 2 * r; k += kColTY)
        tile[k * kColTX + threadIdx.x] = float_of_u8(scratch[(long long)clampi(y0 - r + k, 0, H - 1) * sp + xg]);
    __syncthreads();
    const int ly = threadIdx.y * kColRPT;
    float acc[kColRPT];
#pragma unroll
    for (int j = 0; j < kColRPT; ++j) acc[j] = 0.0f;
    const float* col = tile + ly * kColTX + threadIdx.x;
    for (int i = 0; i < taps; ++i) {
        const float k = kw[i];
#pragma unroll
        for (int j = 0; j < kColRPT; ++j) acc[j] = __fadd_rn(acc[j], __fmul_rn(col[(i + j) * kColTX], k));
    }
    const int x = x0 + threadIdx.x;
    if (x >= W) return;
#pragma unroll
    for (int j = 0; j < kColRPT; ++j) {
        const int y = y0 + ly + j;
        if (y < H) dst[(long long)y * dst_stride + x] = (uint8_t)clamp_u8(acc[j]);
    }
}

// imageproc's kernel for sigma, built in f32 with each operation rounded
// separately (this file's host code is compiled with -ffp-contract=off); the
// same values as the engine's blur tables.
int gaussian_taps(float sigma, BlurTaps* t) {
    const float fr = std::ceil(2.0f * sigma);
    // compared as a float first: a radius beyond int range must not reach the cast
    if (!(fr <= (float)kMaxRadius)) return -1;
    const int r = fr > 0.0f ? (int)fr : 0;
    const float c = 1.0f / (std::sqrt(2.0f * 3.14159265358979323846f) * sigma);
    t->r = r;
    for (int i = 0; i < kTapSlots; ++i) t->w[i] = 0.0f;
    for (int i = 0; i <= r; ++i) {
        const float x = (float)i;
        const float v = c * std::exp(-(x * x) / (2.0f * (sigma * sigma)));
        t->w[r + i] = v;
        t->w[r - i] = v;
    }
    return 0;
}

std::mutex g_scratch_mu;
void* g_scratch_ptr[kMaxDevices] = {};

// Device address of g_blur_scratch on the current device, looked up on first
// use with that device current.
int scratch_address(uint8_t** out) {
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return report_error(SIFT_CUDA_ERR_CUDA, cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices)
        return report_error(SIFT_CUDA_ERR_UNSUPPORTED, "sift_cuda_gaussian_blur_u8_noalloc: device ordinal above 63");
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    if (!g_scratch_ptr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_blur_scratch);
        if (e != cudaSuccess || !p) {
            char msg[160];
            std::snprintf(msg, sizeof msg, "sift_cuda_gaussian_blur_u8_noalloc: cudaGetSymbolAddress failed: %s",
                          cudaGetErrorString(e));
            return report_error(SIFT_CUDA_ERR_CUDA, msg);
        }
        g_scratch_ptr[dev] = p;
    }
    *out = (uint8_t*)g_scratch_ptr[dev];
    return 0;
}

}  // namespace
}  // namespace sift

extern "C" int sift_cuda_gaussian_blur_u8_noalloc(const uint8_t* d_src, uint32_t width, uint32_t height,
                                                  uint32_t src_stride, uint8_t* d_dst, uint32_t dst_stride,
                                                  float sigma, void* stream) {
    using namespace sift;
    if (width == 0 || height == 0) return 0;
    if (!d_src || !d_dst || src_stride < width || dst_stride < width)
        return report_error(SIFT_CUDA_ERR_INVALID_ARGUMENT,
                            "sift_cuda_gaussian_blur_u8_noalloc: NULL image pointer or stride < width");
    if (!(sigma > 0.0f) || !std::isfinite(sigma))
        return report_error(SIFT_CUDA_ERR_INVALID_ARGUMENT, "sift_cuda_gaussian_blur_u8_noalloc: sigma must be > 0");
    const size_t sp = ((size_t)width + 15) & ~(size_t)15;
    if (width > (uint32_t)kMaxWidth || sp * height > kScratchBytes) {
        char msg[200];
        std::snprintf(msg, sizeof msg,
                      "sift_cuda_gaussian_blur_u8_noalloc: a %u x %u image needs %zu bytes of scratch; the limit is "
                      "%zu bytes and width <= %d",
                      width, height, sp * height, kScratchBytes, kMaxWidth);
        return report_error(SIFT_CUDA_ERR_UNSUPPORTED, msg);
    }
    BlurTaps taps;
    if (gaussian_taps(sigma, &taps))
        return report_error(SIFT_CUDA_ERR_UNSUPPORTED,
                            "sift_cuda_gaussian_blur_u8_noalloc: the kernel radius ceil(2 sigma) is above 64");
    uint8_t* scratch = nullptr;
    if (int rc = scratch_address(&scratch)) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    const int W = (int)width, H = (int)height, r = taps.r;
    const size_t rows_smem = sizeof(float) * ((size_t)kTapSlots + 1 + (size_t)W + 2 * (size_t)r + 3);
    const size_t cols_smem = sizeof(float) * ((size_t)kTapSlots + 1 + (size_t)(kColRows + 2 * r) * kColTX);
    k_rows_to_scratch<<<H, kRowThreads, rows_smem, st>>>(d_src, (long long)src_stride, scratch, (int)sp, W, taps);
    dim3 grid((W + kColTX - 1) / kColTX, (H + kColRows - 1) / kColRows);
    k_cols_from_scratch<<<grid, dim3(kColTX, kColTY), cols_smem, st>>>(scratch, (int)sp, d_dst,
                                                                      (long long)dst_stride, W, H, taps);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        char msg[160];
        std::snprintf(msg, sizeof msg, "sift_cuda_gaussian_blur_u8_noalloc: launch failed: %s", cudaGetErrorString(e));
        return report_error(SIFT_CUDA_ERR_CUDA, msg);
    }
    return 0;
}
