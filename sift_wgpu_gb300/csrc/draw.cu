// draw.cu — draw_keypoints_to_image (src/lib.rs:69-116) on the device: the
// grey image as RGB (to_rgb8 replicates the grey value), then for every
// keypoint a filled circle of radius 6 at (x as i32, y as i32), its
// orientation line from (x, y) to (x + 6 cos a, y + 6 sin a) and a filled
// circle of radius 1, all in one colour. Every write is the same colour, so
// the image is the union of the drawn pixel sets whatever the order: one
// thread per keypoint, overlapping writes store equal bytes.
//
// The primitives restate imageproc 0.25.0 (not vendored; Cargo.lock:634-636):
// draw_filled_circle_mut as the midpoint-circle walk that fills horizontal
// spans through draw_line_segment_mut, and draw_line_segment_mut as a
// Bresenham walk over f32 endpoints with an f32 error term, each point kept if
// it lies inside the image.
#include "sift_internal.cuh"

namespace sift {
namespace {

struct Rgb {
    uint8_t r, g, b;
};

__device__ __forceinline__ void put(uint8_t* img, int pitch, int W, int H, int x, int y, Rgb c) {
    if (x < 0 || x >= W || y < 0 || y >= H) return;
    uint8_t* p = img + (long long)y * pitch + 3 * x;
    p[0] = c.r;
    p[1] = c.g;
    p[2] = c.b;
}

// BresenhamLineIter over f32 endpoints (coordinates truncated with `as i32`).
__device__ void line(uint8_t* img, int pitch, int W, int H, float x0, float y0, float x1, float y1, Rgb c) {
    const bool steep = fabsf(__fsub_rn(y1, y0)) > fabsf(__fsub_rn(x1, x0));
    if (steep) {
        float t = x0;
        x0 = y0;
        y0 = t;
        t = x1;
        x1 = y1;
        y1 = t;
    }
    if (x0 > x1) {
        float t = x0;
        x0 = x1;
        x1 = t;
        t = y0;
        y0 = y1;
        y1 = t;
    }
    const float dx = __fsub_rn(x1, x0), dy = fabsf(__fsub_rn(y1, y0));
    int x = rust_as_i32(x0), y = rust_as_i32(y0);
    const int end_x = rust_as_i32(x1), y_step = y0 < y1 ? 1 : -1;
    float err = __fdiv_rn(dx, 2.0f);
    for (int guard = 0; x <= end_x && guard < 4096; ++guard) {
        if (steep)
            put(img, pitch, W, H, y, x, c);
        else
            put(img, pitch, W, H, x, y, c);
        ++x;
        err = __fsub_rn(err, dy);
        if (err < 0.0f) {
            y += y_step;
            err = __fadd_rn(err, dx);
        }
    }
}

// draw_filled_circle_mut: midpoint circle, four horizontal spans per step.
__device__ void filled_circle(uint8_t* img, int pitch, int W, int H, int cx, int cy, int radius, Rgb c) {
    int x = 0, y = radius, p = 1 - radius;
    while (x <= y) {
        line(img, pitch, W, H, (float)(cx - x), (float)(cy + y), (float)(cx + x), (float)(cy + y), c);
        line(img, pitch, W, H, (float)(cx - y), (float)(cy + x), (float)(cx + y), (float)(cy + x), c);
        line(img, pitch, W, H, (float)(cx - x), (float)(cy - y), (float)(cx + x), (float)(cy - y), c);
        line(img, pitch, W, H, (float)(cx - y), (float)(cy - x), (float)(cx + y), (float)(cy - x), c);
        ++x;
        if (p < 0) {
            p += 2 * x + 1;
        } else {
            --y;
            p += 2 * (x - y) + 1;
        }
    }
}

__global__ void k_gray_to_rgb(const uint8_t* __restrict__ gray, int stride, uint8_t* __restrict__ rgb, int pitch,
                              int W, int H) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
    if (x >= W || y >= H) return;
    const uint8_t v = gray[(long long)y * stride + x];
    uint8_t* p = rgb + (long long)y * pitch + 3 * x;
    p[0] = v;
    p[1] = v;
    p[2] = v;
}

__global__ void k_draw_keypoints(const Keypoint* __restrict__ kps, uint32_t n, uint8_t* rgb, int pitch, int W, int H,
                                 Rgb c) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const Keypoint k = kps[i];
    // size is fixed at 2.0 in the reference: radius round(2 * 3) = 6, at least 2
    const int radius = 6;
    const int cx = rust_as_i32(k.x), cy = rust_as_i32(k.y);
    filled_circle(rgb, pitch, W, H, cx, cy, radius, c);
    // cos / sin correctly rounded to f32
    const float ca = (float)cos((double)k.angle), sa = (float)sin((double)k.angle);
    const float xe = __fadd_rn(k.x, __fmul_rn((float)radius, ca)), ye = __fadd_rn(k.y, __fmul_rn((float)radius, sa));
    line(rgb, pitch, W, H, k.x, k.y, xe, ye, c);
    filled_circle(rgb, pitch, W, H, cx, cy, 1, c);
}

}  // namespace

int launch_draw_keypoints(const uint8_t* d_gray, int stride, const Keypoint* d_kps, uint32_t n, uint8_t* d_rgb,
                          int pitch, int W, int H, uint8_t r, uint8_t g, uint8_t b, cudaStream_t st) {
    if (W <= 0 || H <= 0) return 0;
    k_gray_to_rgb<<<dim3((W + 255) / 256, H), 256, 0, st>>>(d_gray, stride, d_rgb, pitch, W, H);
    if (n) k_draw_keypoints<<<(n + 127) / 128, 128, 0, st>>>(d_kps, n, d_rgb, pitch, W, H, Rgb{r, g, b});
    return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace sift
