// convert.cu — colour pixels to the engine's 8-bit luma input, on the device.
//
// The reference turns its input into GrayImage before the pyramid
// (img.to_luma8(), src/sift.rs:1202 and 1256-1258) and, in its WASM entry,
// converts canvas RGBA itself (img_from_raw, src/wasm.rs:79-104). Both run
// here as one pass over the colour image already in device memory, writing
// the engine's image plane:
//
//   SIFT_CUDA_PIXELS_RGB8 / RGBA8   image 0.25.6 to_luma8 (Cargo.lock:634-636,
//       not vendored; restated): l = (2126 r + 7152 g + 722 b) / 10000 in
//       integers, truncating; alpha ignored.
//   SIFT_CUDA_PIXELS_RGBA8_CANVAS   src/wasm.rs:89-93: luma = 0.299 r + 0.587 g
//       + 0.114 b in f32, each product and sum rounded in that order, then
//       `as u8` (truncation toward zero, saturating).
//
// One thread per output pixel, 4 consecutive pixels per thread for the
// 4-channel formats (16-byte loads); the kernel is bound by its HBM bytes
// (3-4 read + 1 written per pixel).
#include <algorithm>

#include "sift_internal.cuh"

namespace sift {
namespace {

__device__ __forceinline__ uint32_t luma_srgb(uint32_t r, uint32_t g, uint32_t b) {
    return (2126u * r + 7152u * g + 722u * b) / 10000u;
}

__device__ __forceinline__ uint32_t luma_canvas(uint32_t r, uint32_t g, uint32_t b) {
    const float l = __fadd_rn(__fadd_rn(__fmul_rn(0.299f, (float)r), __fmul_rn(0.587f, (float)g)),
                              __fmul_rn(0.114f, (float)b));
    return l >= 255.0f ? 255u : (l > 0.0f ? (uint32_t)l : 0u);
}

template <int FMT>
__global__ void __launch_bounds__(256) k_to_luma(const uint8_t* __restrict__ px, long long stride, int W, int H,
                                                 uint8_t* __restrict__ out, long long out_pitch) {
    chain_wait();
    const int y = blockIdx.y;
    const uint8_t* row = px + (long long)y * stride;
    uint8_t* o = out + (long long)y * out_pitch;
    if (FMT == SIFT_CUDA_PIXELS_RGB8) {
        for (int x = blockIdx.x * blockDim.x + threadIdx.x; x < W; x += gridDim.x * blockDim.x) {
            const uint8_t* p = row + 3 * x;
            o[x] = (uint8_t)luma_srgb(p[0], p[1], p[2]);
        }
        return;
    }
    // 4 channels: 4 pixels (16 bytes) per step when the row allows it
    const bool vec = (stride & 15) == 0 && ((uintptr_t)px & 15) == 0;
    for (int x4 = (blockIdx.x * blockDim.x + threadIdx.x) * 4; x4 < W; x4 += gridDim.x * blockDim.x * 4) {
        uint32_t w[4];
        if (vec && x4 + 4 <= W) {
            const uint4 v = *reinterpret_cast<const uint4*>(row + 4 * x4);
            w[0] = v.x;
            w[1] = v.y;
            w[2] = v.z;
            w[3] = v.w;
        } else {
            for (int k = 0; k < 4; ++k) {
                const int x = min(x4 + k, W - 1);
                const uint8_t* p = row + 4 * x;
                w[k] = p[0] | (p[1] << 8) | (p[2] << 16) | ((uint32_t)p[3] << 24);
            }
        }
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            if (x4 + k >= W) break;
            const uint32_t r = w[k] & 0xffu, g = (w[k] >> 8) & 0xffu, b = (w[k] >> 16) & 0xffu;
            o[x4 + k] = (uint8_t)(FMT == SIFT_CUDA_PIXELS_RGBA8 ? luma_srgb(r, g, b) : luma_canvas(r, g, b));
        }
    }
}

}  // namespace

int pixel_channels(int format) {
    switch (format) {
        case SIFT_CUDA_PIXELS_GRAY8: return 1;
        case SIFT_CUDA_PIXELS_RGB8: return 3;
        case SIFT_CUDA_PIXELS_RGBA8:
        case SIFT_CUDA_PIXELS_RGBA8_CANVAS: return 4;
        default: return 0;
    }
}

int launch_to_luma(int format, const uint8_t* px, long long stride, int W, int H, uint8_t* out, long long out_pitch,
                   cudaStream_t st) {
    if (W <= 0 || H <= 0) return 0;
    const int per = format == SIFT_CUDA_PIXELS_RGB8 ? 1 : 4;
    dim3 grid((unsigned)std::min<long long>(((long long)W + 256 * per - 1) / (256 * per), 64), (unsigned)H);
    switch (format) {
        case SIFT_CUDA_PIXELS_RGB8:
            if (launch_chained(k_to_luma<SIFT_CUDA_PIXELS_RGB8>, grid, 256, 0, st, px, stride, W, H, out,
                               out_pitch) != cudaSuccess)
                return -1;
            break;
        case SIFT_CUDA_PIXELS_RGBA8:
            if (launch_chained(k_to_luma<SIFT_CUDA_PIXELS_RGBA8>, grid, 256, 0, st, px, stride, W, H, out,
                               out_pitch) != cudaSuccess)
                return -1;
            break;
        case SIFT_CUDA_PIXELS_RGBA8_CANVAS:
            if (launch_chained(k_to_luma<SIFT_CUDA_PIXELS_RGBA8_CANVAS>, grid, 256, 0, st, px, stride, W, H, out,
                               out_pitch) != cudaSuccess)
                return -1;
            break;
        default: return -1;
    }
    return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace sift
