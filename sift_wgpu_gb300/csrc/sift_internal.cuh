// sift_internal.cuh — shared types and helpers of the sm_103a SIFT engine.
//
// The whole library is compiled with --fmad=false: the reference computes in
// f32 without fused multiply-add (Rust never contracts), and the pyramid,
// extrema and refinement stages reproduce its results bit for bit only when
// every product and sum is rounded separately. Device code that may fuse uses
// fmaf explicitly.
#pragma once

#include <cuda_runtime.h>
#include <cuda_fp16.h>
#include <stdint.h>

#include "../../include/sift_cuda.h"

namespace sift {

constexpr int kOriBins = 36;            // src/sift.rs:21
constexpr int kOriMaxPeaks = 18;        // strict local maxima of a 36-bin circle
constexpr int kDescBins = 8;            // src/sift.rs:28
constexpr int kDescWidth = 4;           // src/sift.rs:29
constexpr int kDescLen = 128;           // 4 x 4 x 8
constexpr float kPi = 3.14159265358979323846f;
constexpr int kMaxOctaves = 16;

using Keypoint = SiftCudaKeypoint;

// Device counters of one run, zeroed at its start. Each octave has its own
// lists and counters (its detection chain runs as soon as its levels exist);
// the final keypoints of octave o go after those of octaves 0..o-1.
struct OctCounters {
    uint32_t n_cand;    // candidates (find_scale_space_extrema)
    uint32_t n_ref;     // refined keypoints
    uint32_t n_ori;     // oriented keypoints
    uint32_t out_base;  // first output slot of the octave
    uint32_t next_ori;  // work queues of the persistent gather kernels
    uint32_t next_desc;
    uint32_t pad[2];
};

struct Counters {
    uint32_t n_candidates;  // totals (filled by the last octave's chain)
    uint32_t n_refined;
    uint32_t n_oriented;    // keypoints in the output
    uint32_t overflow;      // bit 0 candidates, 2 oriented, 8 a scan wait ran out
    uint32_t pad[4];
    OctCounters oct[kMaxOctaves];
};

// Geometry of one octave of one image in the device arena.
struct OctaveDev {
    int W, H, pitch;          // pitch in elements (G and u8 planes)
    int nw;                   // 32-pixel words per row of the extrema mask
    long long g_off;          // element offset of level 0 in the G arena
    long long plane;          // elements per plane (pitch * H)
    long long word_base;      // first word of this octave in the mask arena
    long long u_off;          // byte offset of level 0 in the u8 level arena
    int octave;               // the octave (keypoint scale 2^octave)
    int image;                // the image of a batch (0 for one image)
    long long t_off;          // byte offset of the entry's horizontal-pass plane (batch runs)
};

// A batch's pyramid in device memory (u8 storage): the entries of the batch
// (image-major), the u8 level arena, the horizontal-pass planes, and the
// input images packed at per-image offsets.
// Where a host call's image is read from, set before each run: the
// engine's device copy, or the caller's pageable buffer on a device that
// reads pageable host memory coherently (the captured graph reads the cell).
struct ImgRef {
    const uint8_t* ptr;
    long long pitch;
};

struct BatchPyr {
    uint8_t* U;
    const OctaveDev* ents;
    int O, S;
    // image k: address of its first byte (the batch's device copy, or the
    // caller's host buffer on a device that reads pageable host memory) and
    // its row pitch in bytes
    const unsigned long long* img_addr;
    const int* img_pitch;
};

// The (image, octave) entries of a run in device memory, image-major
// (entry = image * num_octaves + octave). The detection, orientation and
// descriptor kernels read a keypoint's geometry through its entry: inside a
// run, a keypoint's `octave` field holds its entry index, which equals the
// octave for a single image (a batch's export writes back the octave).
struct EntryTable {
    const OctaveDev* ents;
    int n;  // entries
    int S;  // num_intervals
};

struct PyramidDev {
    int num_octaves;
    int S;                    // num_intervals
    int levels;               // S + 3
    OctaveDev oct[kMaxOctaves];
};

// The interior of a 2x Lanczos3 resize: output columns [x0, x1) and rows
// [y0, y1) read the source from 2 o - 5 with the same kLz2xTaps taps (bit for
// bit the table's), so a tile inside both ranges can take them as constants.
// An empty range disables it.
constexpr int kLz2xTaps = 12;
struct LanczosUniform {
    int x0, x1, y0, y1;
    float wv[kLz2xTaps], wh[kLz2xTaps];
};

// Exact integer rounding on the FMA pipe. Conversions (F2I/I2F/FRND) run on
// the quarter-rate XU pipe; for |x| < 2^22 adding a power of two of the right
// size in a directed rounding mode leaves the rounded value in the low
// mantissa bits, exactly.
//   floor:  RD(x + 1.5*2^23) - 1.5*2^23   (1.5*2^23 keeps negatives in the binade)
//   trunc:  RZ(x + 2^23) - 2^23           (x >= 0)
constexpr float kMagic = 8388608.0f;         // 2^23
constexpr float kMagic15 = 12582912.0f;      // 1.5 * 2^23
__device__ __forceinline__ float floor_fi(float x, int* xi) {
    const float t = __fadd_rd(x, kMagic15);
    *xi = __float_as_int(t) - 0x4B400000;
    return __fsub_rn(t, kMagic15);
}
__device__ __forceinline__ int floor_i(float x) { return __float_as_int(__fadd_rd(x, kMagic15)) - 0x4B400000; }
__device__ __forceinline__ float trunc_pos(float x) { return __fsub_rn(__fadd_rz(x, kMagic), kMagic); }
// integer value of a float holding an integer in [0, 2^23)
__device__ __forceinline__ int int_of(float v) { return __float_as_int(__fadd_rn(v, kMagic)) - 0x4B000000; }
// u8 -> float without a conversion
__device__ __forceinline__ float float_of_u8(unsigned b) { return __fsub_rn(__uint_as_float(0x4B000000u | b), kMagic); }
// byte K of w -> float: one byte permute assembles the bits 0x4B0000bb (2^23
// + b), one subtraction removes 2^23
template <int K>
__device__ __forceinline__ float float_of_byte(unsigned w) {
    static_assert(K >= 0 && K < 4, "byte index");
    return __fsub_rn(__uint_as_float(__byte_perm(w, 0x4Bu, 0x4550u | K)), kMagic);
}
// round half away from zero (f32::round) to int, |x| < 2^22
__device__ __forceinline__ int round_away_i(float x) {
    const int m = floor_i(__fadd_rn(fabsf(x), 0.5f));
    return x < 0.0f ? -m : m;
}

// v / 255 correctly rounded (the IEEE division) for integer-valued v in
// [0, 255], without a divide: q = v * fl(1/255) and one fused correction step
// q + fl(v - 255 q) * fl(1/255) (the reciprocal-then-residual scheme of
// Markstein, IBM J. Res. Dev. 34(1), 1990). Checked against v / 255 in exact
// rational arithmetic for all 256 inputs.
constexpr float kInv255 = 0.003921568859368563f;  // fl(1/255) = 0x3B808081
__device__ __forceinline__ float div255(float v) {
    const float q = __fmul_rn(v, kInv255);
    return __fmaf_rn(__fmaf_rn(-q, 255.0f, v), kInv255, q);
}

// imageproc's Clamp<f32> for u8 on the truncation path, as a float:
// min(max(trunc(a), 0), 255) (trunc of a negative a is <= 0).
__device__ __forceinline__ float clamp_u8f(float a) { return fminf(fmaxf(trunc_pos(a), 0.0f), 255.0f); }

// f32 -> u8 the way imageproc's Clamp<f32> for u8 does it: truncation of
// values strictly inside (0, 255), saturation outside.
__device__ __forceinline__ int clamp_u8(float a) {
    if (a < 255.0f) {
        if (a > 0.0f) return (int)a;
        return 0;
    }
    return 255;
}

__device__ __forceinline__ int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

// `f as i32` in Rust: saturating, NaN -> 0.
__device__ __forceinline__ int rust_as_i32(float v) {
    if (v != v) return 0;
    if (v >= 2147483648.0f) return 2147483647;
    if (v <= -2147483648.0f) return (-2147483647 - 1);
    return (int)v;
}

// f32::rem_euclid
__device__ __forceinline__ float rem_euclid(float a, float b) {
    float r = fmodf(a, b);
    return r < 0.0f ? __fadd_rn(r, fabsf(b)) : r;
}

// f32::rem_euclid(a, b) for b > 0 and |a| < 2b, without the general fmodf:
// there fmod(a, b) is a when |a| < b and a - copysign(b, a) otherwise, a
// subtraction that is exact (Sterbenz), so the result is bit-identical.
__device__ __forceinline__ float rem_euclid_2b(float a, float b) {
    const float r = fabsf(a) < b ? a : __fsub_rn(a, copysignf(b, a));
    return r < 0.0f ? __fadd_rn(r, b) : r;
}

// atan2 for the descriptor's gradient angles, written for this engine:
// octant reduction to a = min(|x|,|y|) / max(|x|,|y|) in [0, 1], then
// atan(a) = a * P(a^2) with P of degree 7, minimax in relative error on
// [0, 1] (Lawson's reweighted least squares; tests/golden/fit_atan2.py makes
// the coefficients; 2.5e-7 relative error evaluated in f32), then the octant
// fix-ups: within 4 ulp of atan2f (tests/test_atan2_gpu.py). atan2(0, 0) = 0. Used where the
// angle is interpolated linearly (descriptor bins), and by the orientation
// histogram, whose bins are a hard floor, only away from the bin edges.
__device__ __forceinline__ float atan2_poly(float y, float x) {
    const float ax = fabsf(x), ay = fabsf(y);
    const float mx = fmaxf(ax, ay), mn = fminf(ax, ay);
    const float a = mx > 0.0f ? __fdividef(mn, mx) : 0.0f;
    const float t = a * a;
    float p = -0.004693340510129929f;
    p = fmaf(p, t, 0.024252643808722496f);
    p = fmaf(p, t, -0.0594867542386055f);
    p = fmaf(p, t, 0.09914319962263107f);
    p = fmaf(p, t, -0.14019492268562317f);
    p = fmaf(p, t, 0.19969725608825684f);
    p = fmaf(p, t, -0.33331990242004395f);
    p = fmaf(p, t, 0.9999998807907104f);
    float r = p * a;
    if (ay > ax) r = 1.5707963705062866f - r;
    if (x < 0.0f) r = 3.1415927410125732f - r;
    return copysignf(r, y);
}

// atan2_poly of two gradients at once: the same operations on f32x2 pairs
// (each element rounds as the scalar ones do); a = min * rcp(max) by the
// hardware reciprocal, the form __fdividef takes for these arguments, so the
// results equal atan2_poly's (tests/test_atan2_gpu.py).
// the hardware's approximate reciprocal (one instruction)
__device__ __forceinline__ float rcp_approx(float x) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ float2 atan2_poly2(float2 y, float2 x) {
    const float ax0 = fabsf(x.x), ay0 = fabsf(y.x), ax1 = fabsf(x.y), ay1 = fabsf(y.y);
    const float mx0 = fmaxf(ax0, ay0), mx1 = fmaxf(ax1, ay1);
    const float2 mn = make_float2(fminf(ax0, ay0), fminf(ax1, ay1));
    float2 a = __fmul2_rn(mn, make_float2(rcp_approx(mx0), rcp_approx(mx1)));
    a.x = mx0 > 0.0f ? a.x : 0.0f;
    a.y = mx1 > 0.0f ? a.y : 0.0f;
    const float2 t = __fmul2_rn(a, a);
    float2 p = __ffma2_rn(make_float2(-0.004693340510129929f, -0.004693340510129929f), t,
                          make_float2(0.024252643808722496f, 0.024252643808722496f));
    p = __ffma2_rn(p, t, make_float2(-0.0594867542386055f, -0.0594867542386055f));
    p = __ffma2_rn(p, t, make_float2(0.09914319962263107f, 0.09914319962263107f));
    p = __ffma2_rn(p, t, make_float2(-0.14019492268562317f, -0.14019492268562317f));
    p = __ffma2_rn(p, t, make_float2(0.19969725608825684f, 0.19969725608825684f));
    p = __ffma2_rn(p, t, make_float2(-0.33331990242004395f, -0.33331990242004395f));
    p = __ffma2_rn(p, t, make_float2(0.9999998807907104f, 0.9999998807907104f));
    float2 r = __fmul2_rn(p, a);
    const float2 neg1 = make_float2(-1.0f, -1.0f);
    const float2 r2 = __ffma2_rn(r, neg1, make_float2(1.5707963705062866f, 1.5707963705062866f));
    r.x = ay0 > ax0 ? r2.x : r.x;
    r.y = ay1 > ax1 ? r2.y : r.y;
    const float2 r4 = __ffma2_rn(r, neg1, make_float2(3.1415927410125732f, 3.1415927410125732f));
    r.x = x.x < 0.0f ? r4.x : r.x;
    r.y = x.y < 0.0f ? r4.y : r.y;
    return make_float2(copysignf(r.x, y.x), copysignf(r.y, y.y));
}

// atan2(y, x) in units of 45-degree bins (pi/4 = 1), in [-4, 4]: a = min/max
// of |x|, |y| and an odd degree-9 polynomial a * P(a^2), minimax in absolute
// error against atan(a) * 4/pi on [0, 1] (tests/golden/fit_atan2.py; max
// error 1.5e-5 bin), then the octant fix-ups. For sums that are
// interpolated linearly into bins (the descriptor), not for exact angles.
__device__ __forceinline__ float atan2_bins(float y, float x) {
    const float ax = fabsf(x), ay = fabsf(y);
    const float mx = fmaxf(ax, ay), mn = fminf(ax, ay);
    const float a = mx > 0.0f ? __fdividef(mn, mx) : 0.0f;
    const float t = a * a;
    float p = 0.02654082328081131f;
    p = fmaf(p, t, -0.10842443257570267f);
    p = fmaf(p, t, 0.22938594222068787f);
    p = fmaf(p, t, -0.4205571115016937f);
    p = fmaf(p, t, 1.2730693817138672f);
    float r = p * a;
    if (ay > ax) r = 2.0f - r;
    if (x < 0.0f) r = 4.0f - r;
    return copysignf(r, y);
}

// atan2_bins of two gradients at once: the same polynomial and octant
// fix-ups evaluated on f32x2 pairs (each element rounds as the scalar
// operations do), with a = min * rcp(max) by the hardware reciprocal, so the
// same error bound (tests/test_atan2_gpu.py).
__device__ __forceinline__ float2 atan2_bins2(float2 y, float2 x) {
    const float ax0 = fabsf(x.x), ay0 = fabsf(y.x), ax1 = fabsf(x.y), ay1 = fabsf(y.y);
    const float2 mx = make_float2(fmaxf(ax0, ay0), fmaxf(ax1, ay1));
    const float2 mn = make_float2(fminf(ax0, ay0), fminf(ax1, ay1));
    // max(mx, 1e-30): atan2(0, 0) = 0 * 1e30 = 0
    const float2 a =
        __fmul2_rn(mn, make_float2(rcp_approx(fmaxf(mx.x, 1e-30f)), rcp_approx(fmaxf(mx.y, 1e-30f))));
    const float2 t = __fmul2_rn(a, a);
    float2 p = __ffma2_rn(make_float2(0.02654082328081131f, 0.02654082328081131f), t,
                          make_float2(-0.10842443257570267f, -0.10842443257570267f));
    p = __ffma2_rn(p, t, make_float2(0.22938594222068787f, 0.22938594222068787f));
    p = __ffma2_rn(p, t, make_float2(-0.4205571115016937f, -0.4205571115016937f));
    p = __ffma2_rn(p, t, make_float2(1.2730693817138672f, 1.2730693817138672f));
    float2 r = __fmul2_rn(p, a);
    const float2 neg1 = make_float2(-1.0f, -1.0f);
    const float2 r2 = __ffma2_rn(r, neg1, make_float2(2.0f, 2.0f));
    r.x = ay0 > ax0 ? r2.x : r.x;
    r.y = ay1 > ax1 ? r2.y : r.y;
    const float2 r4 = __ffma2_rn(r, neg1, make_float2(4.0f, 4.0f));
    r.x = x.x < 0.0f ? r4.x : r.x;
    r.y = x.y < 0.0f ? r4.y : r.y;
    return make_float2(copysignf(r.x, y.x), copysignf(r.y, y.y));
}

// The hardware's approximate square root and base-2 exponential (one
// instruction each; subnormal inputs and results flush to zero).
__device__ __forceinline__ float sqrt_approx(float x) {
    float r;
    asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ float ex2_approx(float x) {
    float r;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// Chained launches (programmatic dependent launch). The pipeline's kernels
// go out with launch_chained, and every one of them starts with chain_wait:
// griddepcontrol.wait holds the grid until the previous grid in its stream
// has completed and its memory is visible, so nothing is read or overwritten
// early. No kernel signals launch_dependents, so a grid's dependents are
// released as its CTAs exit: the next launch overlaps the previous grid's
// tail instead of following its completion, without holding SM slots while
// it waits. (Released at the start instead, waiting CTAs of one octave's
// chain took slots from the other octaves' kernels: 1080p 2057 vs 2209
// images/s, although 512^2 rose to 4932.) For kernels launched normally the
// wait does nothing.
__device__ __forceinline__ void chain_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

template <typename... KArgs, typename... Args>
inline cudaError_t launch_chained(void (*k)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                                  Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k, static_cast<KArgs>(args)...);
}

// Scan helpers (scan.cu).
enum ScanInput { SCAN_U32 = 0, SCAN_POPC = 1 };
// Exclusive scan of n values in one launch (n_dev, when not null, overrides n
// at run time and must be <= n). total_out receives the sum. state holds
// scan_state_words(n) 64-bit words that must be zero when the scan starts;
// a look-back wait that runs out sets bit 8 of *err.
size_t scan_state_words(size_t n);
int scan_exclusive(const uint32_t* in, ScanInput mode, uint32_t* out, size_t n, const uint32_t* n_dev,
                   uint32_t* total_out, unsigned long long* state, uint32_t* err, cudaStream_t st);

}  // namespace sift
