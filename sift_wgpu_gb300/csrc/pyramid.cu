// pyramid.cu — Gaussian pyramid kernels (sm_103a).
//
// Stage (a) of the hot path: generate_gaussian_pyramid and
// generate_dog_pyramid (src/sift.rs:129-204), with the base blur of
// detect_and_compute_cpu (src/sift.rs:1200-1214). The levels are
// reference-compatible: each separable blur pass and the Lanczos3 resize end
// in u8 values exactly as the reference's GrayImage levels do, so every level
// is bit-identical to the CPU path, and so is every DoG value the detection
// forms from them. Products and sums are rounded one by one
// (__fmul_rn/__fadd_rn) in the reference's tap order.
//
// Every level is written as its u8 plane (1 byte/pixel, what the next level,
// the resize and every later stage read; DoG is formed from it where it is
// read, never stored) and, in the f32 and f16 storage modes, also in that
// type (f32 v/255 or f16 v, read by orientation and descriptors); the default
// u8 storage writes the u8 plane alone. Nothing in the chain re-reads a
// 4-byte plane.
//
// Kernels
//   k_blur_level   both separable passes of a level for r <= 8 (the first two
//                  octaves at the default sigma): a 64 x 64 tile stages its
//                  u8 window with 16-byte loads, the horizontal pass goes to
//                  shared memory, the vertical pass writes level and u8.
//   k_blur_rows    horizontal pass for larger radii, one row per CTA. u8 out.
//   k_blur_cols    vertical pass for larger radii on a 32 x 64 tile.
//   k_lanczos_fused  the 2x Lanczos3 resize between octaves, both passes.
// The base level of a host call reads its image through an ImgRef cell (the
// engine's device copy, or the caller's pageable buffer in place).
#include <cstring>
#include <type_traits>

#include "sift_internal.cuh"

namespace sift {
namespace {

// v / 255 in f32, the IEEE quotient the reference computes (div255: a
// multiply and one fused correction, exact for every u8 value).
__device__ __forceinline__ float norm255(int v) { return div255((float)v); }

// Level storage: f32 holds v/255 (the reference's convert_u8_to_f32_gray
// value, src/sift.rs:92-101), f16 holds v (v/255 is not exact in f16), u8
// storage stores nothing beyond the u8 plane.
template <typename T>
__device__ __forceinline__ void store_level(T* p, int v, float vn);
template <>
__device__ __forceinline__ void store_level<float>(float* p, int v, float vn) {
    *p = vn;
}
template <>
__device__ __forceinline__ void store_level<__half>(__half* p, int v, float) {
    *p = __int2half_rn(v);
}
// u8 storage: the level is its u8 plane, which every kernel writes anyway
template <>
__device__ __forceinline__ void store_level<uint8_t>(uint8_t*, int, float) {}

__device__ __forceinline__ void unpack16(const uint4 b, float* v) {
    const unsigned w[4] = {b.x, b.y, b.z, b.w};
#pragma unroll
    for (int e = 0; e < 4; ++e) {
        v[4 * e + 0] = float_of_byte<0>(w[e]);
        v[4 * e + 1] = float_of_byte<1>(w[e]);
        v[4 * e + 2] = float_of_byte<2>(w[e]);
        v[4 * e + 3] = float_of_byte<3>(w[e]);
    }
}

// imageproc's f32 -> u8 clamp (truncation) as an int
__device__ __forceinline__ int to_u8(float a) { return int_of(clamp_u8f(a)); }

constexpr int kRowThreads = 128;

// One row per CTA. Shared layout: weights[taps] (padded to a multiple of 4),
// then the row with r clamp-to-edge pixels on each side and 8 floats of slack.
__device__ __forceinline__ void blur_row(const uint8_t* __restrict__ in, int in_pitch, uint8_t* __restrict__ out,
                                         int out_pitch, int W, int r, const float* __restrict__ wts, int y, float* sm) {
    const int taps = 2 * r + 1;
    const int wpad = (taps + 3) & ~3;
    float* kw = sm;
    float* row = sm + wpad;
    const uint8_t* src = in + (long long)y * in_pitch;
    for (int i = threadIdx.x; i < wpad; i += blockDim.x) kw[i] = i < taps ? wts[i] : 0.0f;
    const int padded = W + 2 * r;
    // Interior as 4-byte words, consecutive lanes on consecutive words: the
    // four stores of a lane land 4 floats apart from its neighbour's (4-way
    // bank sharing; 16-byte words per lane would put a warp's stores in two
    // banks).
    const int nw4 = (in_pitch & 3) == 0 ? (W >> 2) : 0;
#pragma unroll 4
    for (int k = threadIdx.x; k < nw4; k += blockDim.x) {
        const unsigned b = *reinterpret_cast<const unsigned*>(src + 4 * k);
        float* d = row + r + 4 * k;
        d[0] = float_of_byte<0>(b);
        d[1] = float_of_byte<1>(b);
        d[2] = float_of_byte<2>(b);
        d[3] = float_of_byte<3>(b);
    }
    // clamp-to-edge borders, the tail after the whole words and the slack
    const int hi0 = r + 4 * nw4, nb = r + (padded + 8 - hi0);
    for (int j = threadIdx.x; j < nb; j += blockDim.x) {
        const int jj = j < r ? j : hi0 + (j - r);
        row[jj] = float_of_u8(src[clampi(jj - r, 0, W - 1)]);
    }
    __syncthreads();
    uint8_t* dst = out + (long long)y * out_pitch;
    for (int x0 = threadIdx.x * 4; x0 < W; x0 += blockDim.x * 4) {
        float a0 = 0.0f, a1 = 0.0f, a2 = 0.0f, a3 = 0.0f;
        const float* base = row + x0;  // x0 % 4 == 0 and wpad % 4 == 0: 16-byte aligned
        float4 A = *reinterpret_cast<const float4*>(base);
        int i = 0;
        for (; i + 4 <= taps; i += 4) {
            const float4 B = *reinterpret_cast<const float4*>(base + i + 4);
            const float4 K = *reinterpret_cast<const float4*>(kw + i);
            a0 = __fadd_rn(a0, __fmul_rn(A.x, K.x));
            a1 = __fadd_rn(a1, __fmul_rn(A.y, K.x));
            a2 = __fadd_rn(a2, __fmul_rn(A.z, K.x));
            a3 = __fadd_rn(a3, __fmul_rn(A.w, K.x));
            a0 = __fadd_rn(a0, __fmul_rn(A.y, K.y));
            a1 = __fadd_rn(a1, __fmul_rn(A.z, K.y));
            a2 = __fadd_rn(a2, __fmul_rn(A.w, K.y));
            a3 = __fadd_rn(a3, __fmul_rn(B.x, K.y));
            a0 = __fadd_rn(a0, __fmul_rn(A.z, K.z));
            a1 = __fadd_rn(a1, __fmul_rn(A.w, K.z));
            a2 = __fadd_rn(a2, __fmul_rn(B.x, K.z));
            a3 = __fadd_rn(a3, __fmul_rn(B.y, K.z));
            a0 = __fadd_rn(a0, __fmul_rn(A.w, K.w));
            a1 = __fadd_rn(a1, __fmul_rn(B.x, K.w));
            a2 = __fadd_rn(a2, __fmul_rn(B.y, K.w));
            a3 = __fadd_rn(a3, __fmul_rn(B.z, K.w));
            A = B;
        }
        for (; i < taps; ++i) {
            const float k = kw[i];
            a0 = __fadd_rn(a0, __fmul_rn(base[i + 0], k));
            a1 = __fadd_rn(a1, __fmul_rn(base[i + 1], k));
            a2 = __fadd_rn(a2, __fmul_rn(base[i + 2], k));
            a3 = __fadd_rn(a3, __fmul_rn(base[i + 3], k));
        }
        const int v0 = to_u8(a0), v1 = to_u8(a1), v2 = to_u8(a2), v3 = to_u8(a3);
        if (x0 + 3 < W) {  // out_pitch is a multiple of 32 and x0 of 4: one aligned word
            *reinterpret_cast<unsigned*>(dst + x0) =
                (unsigned)v0 | ((unsigned)v1 << 8) | ((unsigned)v2 << 16) | ((unsigned)v3 << 24);
        } else {
            dst[x0] = (uint8_t)v0;
            if (x0 + 1 < W) dst[x0 + 1] = (uint8_t)v1;
            if (x0 + 2 < W) dst[x0 + 2] = (uint8_t)v2;
        }
    }
}

__global__ void __launch_bounds__(kRowThreads) k_blur_rows(const uint8_t* __restrict__ in, int in_pitch,
                                                           uint8_t* __restrict__ out, int out_pitch, int W, int r,
                                                           const float* __restrict__ wts,
                                                           const ImgRef* __restrict__ ref) {
    chain_wait();
    if (ref) {  // a host call's base level: the image is wherever the cell says
        in = ref->ptr;
        in_pitch = (int)ref->pitch;
    }
    extern __shared__ __align__(16) float sm[];
    blur_row(in, in_pitch, out, out_pitch, W, r, wts, blockIdx.x, sm);
}

constexpr int kColTX = 32;                 // output columns per CTA
constexpr int kColRows = 64;               // output rows per CTA
constexpr int kColThreads = 256;           // 8 column groups of 4 x 32 row groups of 2

// Vertical pass over a 32 x 64 output tile. Shared layout: weights padded
// with zeros to a multiple of 8, lut[256] (v / 255 in f32), then
// (64 + taps8 - 1) rows x 32 floats of the u8 intermediate with
// clamp-to-edge rows. Each thread owns 4 columns x 2 rows and slides a
// two-row float4 window down the taps, in unrolled groups of 8; the zero taps
// at the end add +0 to a non-negative sum, which leaves it unchanged. Writes
// level s (TG and u8) as vector stores. No DoG plane is stored: the detection
// stages form DoG(s-1) = G_s/255 - G_{s-1}/255 (src/sift.rs:92-124) from the
// u8 planes through the v / 255 table where they read it.
__host__ __device__ constexpr int taps8(int r) { return ((2 * r + 1) + 7) & ~7; }

template <typename TG>
__device__ __forceinline__ void store_level4(TG* p, const int v[4], const float* lut);

template <typename TG>
__device__ __forceinline__ void blur_cols_tile(const uint8_t* __restrict__ tmp, int tmp_pitch, TG* __restrict__ out,
                                               uint8_t* __restrict__ out_u8, int pitch, int W, int H, int r,
                                               const float* __restrict__ wts, const float* __restrict__ lut255,
                                               int x0, int y0, float* sm) {
    const int taps = 2 * r + 1;
    const int tp = taps8(r);
    float* kw = sm;
    float* lut = sm + tp;
    float* tile = lut + 256;
    const int tid = threadIdx.x;
    for (int i = tid; i < tp; i += kColThreads) kw[i] = i < taps ? wts[i] : 0.0f;
    for (int i = tid; i < 256; i += kColThreads) lut[i] = lut255[i];
    const int rows = kColRows + tp - 1;
    if (x0 + kColTX <= W && (tmp_pitch & 15) == 0) {
        // two 16-byte loads per row, all rows of the tile in flight
#pragma unroll 4
        for (int q = tid; q < rows * 2; q += kColThreads) {
            const int k = q >> 1, h = q & 1;
            const int ys = clampi(y0 - r + k, 0, H - 1);
            float v[16];
            unpack16(*reinterpret_cast<const uint4*>(tmp + (long long)ys * tmp_pitch + x0 + 16 * h), v);
            float* d = tile + k * kColTX + 16 * h;
#pragma unroll
            for (int e = 0; e < 16; ++e) d[e] = v[e];
        }
    } else {
        const int lx = tid & (kColTX - 1);
        const int xg = min(x0 + lx, W - 1);
        for (int k = tid / kColTX; k < rows; k += kColThreads / kColTX) {
            const int ys = clampi(y0 - r + k, 0, H - 1);
            tile[k * kColTX + lx] = float_of_u8(tmp[(long long)ys * tmp_pitch + xg]);
        }
    }
    __syncthreads();
    const int cg = tid & 7, rg = tid >> 3;
    const float4* col = reinterpret_cast<const float4*>(tile) + (2 * rg) * (kColTX / 4) + cg;
    float4 a0 = make_float4(0.0f, 0.0f, 0.0f, 0.0f), a1 = a0;
    float4 w0 = col[0];
    for (int i0 = 0; i0 < tp; i0 += 8) {
        const float4 ka = *reinterpret_cast<const float4*>(kw + i0);
        const float4 kb = *reinterpret_cast<const float4*>(kw + i0 + 4);
        const float k8[8] = {ka.x, ka.y, ka.z, ka.w, kb.x, kb.y, kb.z, kb.w};
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const float4 w1 = col[(i0 + q + 1) * (kColTX / 4)];
            const float k = k8[q];
            a0.x = __fadd_rn(a0.x, __fmul_rn(w0.x, k));
            a0.y = __fadd_rn(a0.y, __fmul_rn(w0.y, k));
            a0.z = __fadd_rn(a0.z, __fmul_rn(w0.z, k));
            a0.w = __fadd_rn(a0.w, __fmul_rn(w0.w, k));
            a1.x = __fadd_rn(a1.x, __fmul_rn(w1.x, k));
            a1.y = __fadd_rn(a1.y, __fmul_rn(w1.y, k));
            a1.z = __fadd_rn(a1.z, __fmul_rn(w1.z, k));
            a1.w = __fadd_rn(a1.w, __fmul_rn(w1.w, k));
            w0 = w1;
        }
    }
    const int xc = x0 + 4 * cg;
    if (xc >= W) return;
    const bool full = xc + 3 < W;
    const float4 acc[2] = {a0, a1};
#pragma unroll
    for (int j = 0; j < 2; ++j) {
        const int y = y0 + 2 * rg + j;
        if (y >= H) break;
        const int v[4] = {to_u8(acc[j].x), to_u8(acc[j].y), to_u8(acc[j].z), to_u8(acc[j].w)};
        const long long o = (long long)y * pitch + xc;
        if (full) {
            store_level4(out + o, v, lut);
            *reinterpret_cast<unsigned*>(out_u8 + o) =
                (unsigned)v[0] | ((unsigned)v[1] << 8) | ((unsigned)v[2] << 16) | ((unsigned)v[3] << 24);
        } else {
            for (int c = 0; c < 4 && xc + c < W; ++c) {
                store_level(out + o + c, v[c], lut[v[c]]);
                out_u8[o + c] = (uint8_t)v[c];
            }
        }
    }
}

template <typename TG>
__global__ void __launch_bounds__(kColThreads) k_blur_cols(const uint8_t* __restrict__ tmp, int tmp_pitch,
                                                          TG* __restrict__ out, uint8_t* __restrict__ out_u8,
                                                          int pitch, int W, int H, int r,
                                                          const float* __restrict__ wts,
                                                          const float* __restrict__ lut255) {
    chain_wait();
    extern __shared__ __align__(16) float sm[];
    blur_cols_tile<TG>(tmp, tmp_pitch, out, out_u8, pitch, W, H, r, wts, lut255, blockIdx.x * kColTX,
                       blockIdx.y * kColRows, sm);
}

// ---------------------------------------------------------------------------
// Packed pairs of f32: mul.rn.f32x2 rounds each of the two products like a
// scalar multiply. The products are added to scalar accumulators: a packed
// multiply followed by a packed add was measured to come out fused (one
// rounding: a third of the sums differed from the reference's), a packed
// multiply followed by scalar adds matched the scalar sequence on 2^20 sums.
typedef unsigned long long f32x2;
__device__ __forceinline__ f32x2 mul2(f32x2 a, f32x2 b) {
    f32x2 d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ f32x2 pack2(float lo, float hi) {
    return ((f32x2)__float_as_uint(hi) << 32) | __float_as_uint(lo);
}
__device__ __forceinline__ float lo2(f32x2 v) { return __uint_as_float((unsigned)v); }
__device__ __forceinline__ float hi2(f32x2 v) { return __uint_as_float((unsigned)(v >> 32)); }
// tap sum step for two accumulators: a + v * k, rounded after the products
// and after the sums
__device__ __forceinline__ void tap2(float& a_lo, float& a_hi, f32x2 v, f32x2 k) {
    const f32x2 p = mul2(v, k);
    a_lo = __fadd_rn(a_lo, lo2(p));
    a_hi = __fadd_rn(a_hi, hi2(p));
}

// ---------------------------------------------------------------------------
// Fused level kernel: both separable passes of one level in one launch, for
// radii up to 8. The CTA stages the (64 + 2r)-row clamp-to-edge neighbourhood
// of its 64 x 64 output tile from the previous level's u8 plane, runs the
// horizontal pass for all 64 + 2r rows into shared memory (u8-truncated like
// imageproc's intermediate image), then the vertical pass, and writes the
// level and its u8 plane; each scale is read once, as bytes.
//
// Staged row layout: shared column c holds global x = x0 - 16 - sh + c with
// sh = r mod 4, so an interior row is the 96 bytes [x0 - 16, x0 + 80) written
// without conditions, and the horizontal pass's first input (x0 - r, column
// 16 + sh - r) is 16-byte aligned for its float4 window. Each vertical-pass
// thread owns 4 columns x 4 rows: one float4 shared load per tap, two packed
// multiplies per row and tap, and vector stores of level and u8 copy.
constexpr int kFTX = 64, kFTY = 64, kFThreads = 256;
constexpr int kFMaxR = 8;
constexpr int kFSW = 100;  // staged row stride (floats): sh + 96 <= 99

size_t blur_fused_smem(int r, int ty = kFTY) {
    const int taps = 2 * r + 1;
    const size_t rows = (size_t)ty + 2 * r;
    return sizeof(float) * ((size_t)3 * ((taps + 3) & ~3) + 256 + rows * kFSW + rows * kFTX);
}

template <typename TG>
__device__ __forceinline__ void store_level4(TG* p, const int v[4], const float* lut);
template <>
__device__ __forceinline__ void store_level4<float>(float* p, const int v[4], const float* lut) {
    *reinterpret_cast<float4*>(p) = make_float4(lut[v[0]], lut[v[1]], lut[v[2]], lut[v[3]]);
}
template <>
__device__ __forceinline__ void store_level4<uint8_t>(uint8_t*, const int*, const float*) {}
template <>
__device__ __forceinline__ void store_level4<__half>(__half* p, const int v[4], const float*) {
    const __half2 a = __halves2half2(__int2half_rn(v[0]), __int2half_rn(v[1]));
    const __half2 b = __halves2half2(__int2half_rn(v[2]), __int2half_rn(v[3]));
    uint2 u;
    u.x = *reinterpret_cast<const unsigned*>(&a);
    u.y = *reinterpret_cast<const unsigned*>(&b);
    *reinterpret_cast<uint2*>(p) = u;
}

// Shared layout of the fused level kernel (floats): kw2[wpad] (pairs),
// kw[wpad], lut[256], src[RH][kFSW] (staged input as floats), hb[RH][kFTX].
// A tile is 64 columns by TY rows (64, or 32 for more, smaller CTAs on small
// planes), computed by 4 * TY threads: 16 per row in the horizontal pass,
// 4 x 4 outputs each in the vertical pass.
template <int R, int TY = kFTY>
struct FusedLayout {
    static_assert(TY == 32 || TY == 64, "fused tile height");
    static constexpr int taps = 2 * R + 1;
    static constexpr int wpad = (taps + 3) & ~3;
    static constexpr int RH = TY + 2 * R;
    static constexpr int sh = R & 3;
    static constexpr int threads = 4 * TY;
};

// the tap weights (single and paired) and the v / 255 table into shared memory
template <int R, int TY = kFTY>
__device__ __forceinline__ void blur_level_weights(const float* __restrict__ wts, const float* __restrict__ lut255,
                                                   float* sm) {
    using Lx = FusedLayout<R, TY>;
    f32x2* kw2 = reinterpret_cast<f32x2*>(sm);
    float* kw = sm + 2 * Lx::wpad;
    float* lut = kw + Lx::wpad;
    for (int i = threadIdx.x; i < Lx::wpad; i += Lx::threads) {
        const float k = i < Lx::taps ? wts[i] : 0.0f;
        kw2[i] = pack2(k, k);
        kw[i] = k;
    }
    for (int i = threadIdx.x; i < 256; i += Lx::threads) lut[i] = lut255[i];
}

template <int R, int TY = kFTY>
__device__ __forceinline__ bool blur_level_interior(int x0, int y0, int W, int H) {
    return x0 >= 16 && x0 + 80 <= W && y0 >= R && y0 + TY + R <= H;
}

// Stages the tile's (TY + 2R)-row neighbourhood from the previous level's u8
// plane (global memory) as floats: interior tiles with 16-byte loads of
// [x0 - 16, x0 + 80), border tiles clamp-to-edge.
template <int R, int TY = kFTY>
__device__ __forceinline__ void blur_level_stage_global(const uint8_t* __restrict__ in, int in_pitch, int W, int H,
                                                        int x0, int y0, float* sm) {
    using Lx = FusedLayout<R, TY>;
    float* src = sm + 3 * Lx::wpad + 256;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (blur_level_interior<R, TY>(x0, y0, W, H) && (in_pitch & 15) == 0) {
        constexpr int Q = 6;
        const uint8_t* org = in + (long long)(y0 - R) * in_pitch + (x0 - 16);
#pragma unroll 2
        for (int q = tid; q < Lx::RH * Q; q += Lx::threads) {
            const int yy = q / Q, k = q - yy * Q;
            float v[16];
            unpack16(*reinterpret_cast<const uint4*>(org + (long long)yy * in_pitch + 16 * k), v);
            float* d = src + (size_t)yy * kFSW + Lx::sh + 16 * k;
#pragma unroll
            for (int e = 0; e < 16; ++e) d[e] = v[e];
        }
    } else {
        // clamp-to-edge, only the columns the passes read: 16 + sh - R .. sh + 80 + R
        for (int yy = warp; yy < Lx::RH; yy += Lx::threads / 32) {
            const uint8_t* row = in + (long long)clampi(y0 - R + yy, 0, H - 1) * in_pitch;
            float* d = src + (size_t)yy * kFSW;
            for (int c = 16 + Lx::sh - R + lane; c <= Lx::sh + 80 + R; c += 32)
                d[c] = float_of_u8(row[clampi(x0 - 16 - Lx::sh + c, 0, W - 1)]);
        }
    }
}

// Both passes from the staged floats (the caller synchronises the CTA
// between staging and this): horizontal pass into hb, then the vertical pass,
// writing the level and its u8 plane.
template <typename TG, int R, int TY = kFTY>
__device__ __forceinline__ void blur_level_compute(TG* __restrict__ out, uint8_t* __restrict__ out_u8, int pitch,
                                                   int W, int H, int x0, int y0, float* sm) {
    using Lx = FusedLayout<R, TY>;
    constexpr int taps = Lx::taps;
    constexpr int RH = Lx::RH;
    constexpr int sh = Lx::sh;
    const f32x2* kw2 = reinterpret_cast<const f32x2*>(sm);
    const float* kw = sm + 2 * Lx::wpad;
    const float* lut = kw + Lx::wpad;
    const float* src = lut + 256;
    float* hb = const_cast<float*>(src) + (size_t)RH * kFSW;
    const int tid = threadIdx.x;
    // horizontal pass: 16 threads per row, 4 outputs each (float4 sliding window)
    {
        const int xq = (tid & 15) * 4;
        for (int yy = tid >> 4; yy < RH; yy += Lx::threads / 16) {
            const float* base = src + (size_t)yy * kFSW + (16 + sh - R) + xq;
            float a0 = 0.0f, a1 = 0.0f, a2 = 0.0f, a3 = 0.0f;
            float4 A = *reinterpret_cast<const float4*>(base);
            int i = 0;
#pragma unroll
            for (; i + 4 <= taps; i += 4) {
                const float4 B = *reinterpret_cast<const float4*>(base + i + 4);
                const float4 K = *reinterpret_cast<const float4*>(kw + i);
                a0 = __fadd_rn(a0, __fmul_rn(A.x, K.x));
                a1 = __fadd_rn(a1, __fmul_rn(A.y, K.x));
                a2 = __fadd_rn(a2, __fmul_rn(A.z, K.x));
                a3 = __fadd_rn(a3, __fmul_rn(A.w, K.x));
                a0 = __fadd_rn(a0, __fmul_rn(A.y, K.y));
                a1 = __fadd_rn(a1, __fmul_rn(A.z, K.y));
                a2 = __fadd_rn(a2, __fmul_rn(A.w, K.y));
                a3 = __fadd_rn(a3, __fmul_rn(B.x, K.y));
                a0 = __fadd_rn(a0, __fmul_rn(A.z, K.z));
                a1 = __fadd_rn(a1, __fmul_rn(A.w, K.z));
                a2 = __fadd_rn(a2, __fmul_rn(B.x, K.z));
                a3 = __fadd_rn(a3, __fmul_rn(B.y, K.z));
                a0 = __fadd_rn(a0, __fmul_rn(A.w, K.w));
                a1 = __fadd_rn(a1, __fmul_rn(B.x, K.w));
                a2 = __fadd_rn(a2, __fmul_rn(B.y, K.w));
                a3 = __fadd_rn(a3, __fmul_rn(B.z, K.w));
                A = B;
            }
#pragma unroll
            for (; i < taps; ++i) {
                const float k = kw[i];
                a0 = __fadd_rn(a0, __fmul_rn(base[i + 0], k));
                a1 = __fadd_rn(a1, __fmul_rn(base[i + 1], k));
                a2 = __fadd_rn(a2, __fmul_rn(base[i + 2], k));
                a3 = __fadd_rn(a3, __fmul_rn(base[i + 3], k));
            }
            const float4 o4 = make_float4(clamp_u8f(a0), clamp_u8f(a1), clamp_u8f(a2), clamp_u8f(a3));
            *reinterpret_cast<float4*>(hb + (size_t)yy * kFTX + xq) = o4;
        }
    }
    __syncthreads();
    // vertical pass: thread = 4 columns x 4 rows, a 4-row float4 window
    // sliding down the taps
    const int cg = tid & 15, rg = tid >> 4;
    const ulonglong2* hb2 = reinterpret_cast<const ulonglong2*>(hb) + cg;  // row stride kFTX / 4
    float4 acc[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[j] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    ulonglong2 w0 = hb2[(4 * rg + 0) * (kFTX / 4)], w1 = hb2[(4 * rg + 1) * (kFTX / 4)],
               w2 = hb2[(4 * rg + 2) * (kFTX / 4)];
#pragma unroll
    for (int i = 0; i < taps; ++i) {
        const ulonglong2 w3 = hb2[(4 * rg + i + 3) * (kFTX / 4)];
        const f32x2 k = kw2[i];
        const ulonglong2 w[4] = {w0, w1, w2, w3};
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            tap2(acc[j].x, acc[j].y, w[j].x, k);
            tap2(acc[j].z, acc[j].w, w[j].y, k);
        }
        w0 = w1;
        w1 = w2;
        w2 = w3;
    }
    const int xc = x0 + 4 * cg;
    if (xc >= W) return;
    const bool full = xc + 3 < W;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const int y = y0 + 4 * rg + j;
        if (y >= H) break;
        const int v[4] = {to_u8(acc[j].x), to_u8(acc[j].y), to_u8(acc[j].z), to_u8(acc[j].w)};
        const long long o = (long long)y * pitch + xc;
        if (full) {
            store_level4(out + o, v, lut);
            *reinterpret_cast<unsigned*>(out_u8 + o) =
                (unsigned)v[0] | ((unsigned)v[1] << 8) | ((unsigned)v[2] << 16) | ((unsigned)v[3] << 24);
        } else {
            for (int c = 0; c < 4 && xc + c < W; ++c) {
                store_level(out + o + c, v[c], lut[v[c]]);
                out_u8[o + c] = (uint8_t)v[c];
            }
        }
    }
}


template <typename TG, int R, int TY = kFTY>
__device__ __forceinline__ void blur_level_tile(const uint8_t* __restrict__ in, int in_pitch, TG* __restrict__ out,
                                                uint8_t* __restrict__ out_u8, int pitch, int W, int H,
                                                const float* __restrict__ wts, const float* __restrict__ lut255,
                                                int x0, int y0, float* sm) {
    static_assert(R >= 1 && R <= kFMaxR, "fused radius");
    blur_level_weights<R, TY>(wts, lut255, sm);
    blur_level_stage_global<R, TY>(in, in_pitch, W, H, x0, y0, sm);
    __syncthreads();
    blur_level_compute<TG, R, TY>(out, out_u8, pitch, W, H, x0, y0, sm);
}

template <typename TG, int R, int TY>
__global__ void __launch_bounds__(4 * TY) k_blur_level(const uint8_t* __restrict__ in, int in_pitch,
                                                          TG* __restrict__ out, uint8_t* __restrict__ out_u8,
                                                          int pitch, int W, int H,
                                                          const float* __restrict__ wts,
                                                          const float* __restrict__ lut255,
                                                          const ImgRef* __restrict__ ref) {
    chain_wait();
    if (ref) {  // a host call's base level: the image is wherever the cell says
        in = ref->ptr;
        in_pitch = (int)ref->pitch;
    }
    extern __shared__ __align__(16) float sm[];
    blur_level_tile<TG, R, TY>(in, in_pitch, out, out_u8, pitch, W, H, wts, lut255, blockIdx.x * kFTX,
                               blockIdx.y * TY, sm);
}

// A level whose blur increment is below 1e-4 is a copy of the previous one
// (src/sift.rs:152-154).
template <typename TG>
__global__ void k_copy_level(const TG* __restrict__ prev, const uint8_t* __restrict__ prev_u8, TG* __restrict__ out,
                             uint8_t* __restrict__ out_u8, int pitch, int W, int H) {
    chain_wait();
    int x = blockIdx.x * blockDim.x + threadIdx.x;
    int y = blockIdx.y;
    if (x >= W) return;
    long long o = (long long)y * pitch + x;
    if constexpr (!std::is_same<TG, uint8_t>::value) out[o] = prev[o];  // u8 storage: out is out_u8
    out_u8[o] = prev_u8[o];
}

// Base level without a blur (sigma <= assumed_blur, src/sift.rs:1204-1214).
template <typename TG>
__global__ void k_u8_to_level(const uint8_t* __restrict__ img, long long stride, TG* __restrict__ out,
                              uint8_t* __restrict__ out_u8, int pitch, int W, int H, const ImgRef* __restrict__ ref) {
    chain_wait();
    if (ref) {
        img = ref->ptr;
        stride = ref->pitch;
    }
    int x = blockIdx.x * blockDim.x + threadIdx.x;
    int y = blockIdx.y;
    if (x >= W) return;
    const int v = (int)img[(long long)y * stride + x];
    const long long o = (long long)y * pitch + x;
    store_level(out + o, v, norm255(v));
    out_u8[o] = (uint8_t)v;
}

// Both Lanczos3 passes of the 2x resize in one kernel (image 0.25.6
// vertical_sample then horizontal_sample): a 32 x 32 output tile stages its
// source window (at most kLzSpan x kLzSpan, checked on the host), runs the
// vertical pass for the columns the horizontal pass reads, then the
// horizontal pass; every value is formed exactly as in the two-kernel form.
// Tiles inside the uniform interior of a 2x resize (LanczosUniform) run both
// passes with the 12 taps as constants: each thread sums 4 outputs from 18
// shared loads, the tap loops unrolled; the sums are the same, in the same
// order.
constexpr int kLzT = 32, kLzSpan = 80, kLzMid = 81;  // odd mid stride: lanes on rows hit 32 banks
constexpr int kLzIn = 96;  // staged row: 16-byte aligned x from x_lo & ~15, x_lo - (x_lo & ~15) + span <= 95

template <typename TG>
__device__ __forceinline__ void lanczos_tile(const uint8_t* __restrict__ src, int src_pitch, TG* __restrict__ dst,
                                             uint8_t* __restrict__ dst_u8, int dst_pitch, int nW, int nH,
                                             const int* __restrict__ vtab, const float* __restrict__ vw,
                                             const int* __restrict__ htab, const float* __restrict__ hw,
                                             const LanczosUniform& uni, int ox0, int oy0) {
    __shared__ __align__(16) float in_rows[kLzSpan][kLzIn];
    __shared__ float mid[kLzT][kLzMid];
    const int* vleft = vtab;
    const int* vcount = vtab + nH;
    const int* voff = vtab + 2 * nH;
    const int* hleft = htab;
    const int* hcount = htab + nW;
    const int* hoff = htab + 2 * nW;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int ox1 = min(ox0 + kLzT, nW), oy1 = min(oy0 + kLzT, nH);
    const int x_lo = hleft[ox0], x_hi = hleft[ox1 - 1] + hcount[ox1 - 1];
    const int y_lo = vleft[oy0], y_hi = vleft[oy1 - 1] + vcount[oy1 - 1];
    const int sw = x_hi - x_lo, sh = y_hi - y_lo;
    // stage: 16-byte words from xa = x_lo & ~15 (staged column c holds x =
    // xa + c; the words end at align16(x_hi) <= the row pitch, a multiple of
    // 32), each byte to a float by one byte permute and one subtraction
    const int xa = x_lo & ~15, xo = x_lo - xa;
    const int nq = (x_hi - xa + 15) >> 4;
    if ((src_pitch & 15) == 0) {
        for (int q = tid; q < sh * nq; q += 256) {
            const int yy = q / nq, k = q - yy * nq;
            float v[16];
            unpack16(*reinterpret_cast<const uint4*>(src + (long long)(y_lo + yy) * src_pitch + xa + 16 * k), v);
            float4* d = reinterpret_cast<float4*>(&in_rows[yy][16 * k]);
#pragma unroll
            for (int e = 0; e < 4; ++e) d[e] = make_float4(v[4 * e], v[4 * e + 1], v[4 * e + 2], v[4 * e + 3]);
        }
    } else {
        for (int q = tid; q < sh * sw; q += 256) {
            const int yy = q / sw, xx = q - yy * sw;
            in_rows[yy][xo + xx] = float_of_u8(src[(long long)(y_lo + yy) * src_pitch + x_lo + xx]);
        }
    }
    __syncthreads();
    // in[y][x]: source (y_lo + y, x_lo + x)
    auto in = [&](int y, int x) -> float { return in_rows[y][xo + x]; };
    if (ox0 >= uni.x0 && ox0 + kLzT <= uni.x1 && oy0 >= uni.y0 && oy0 + kLzT <= uni.y1) {
        // vertical pass: warp w makes mid rows 4w .. 4w+3 from source rows
        // 8w .. 8w+17 (output row r reads from 2r, tap i at j = 2r + i)
        for (int xx = lane; xx < sw; xx += 32) {
            float a[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
            for (int j = 0; j < 18; ++j) {
                const float v = in(8 * warp + j, xx);
#pragma unroll
                for (int r = 0; r < 4; ++r)
                    if (j - 2 * r >= 0 && j - 2 * r < kLz2xTaps) a[r] = __fadd_rn(a[r], __fmul_rn(v, uni.wv[j - 2 * r]));
            }
#pragma unroll
            for (int r = 0; r < 4; ++r) mid[4 * warp + r][xx] = a[r];
        }
        __syncthreads();
        // horizontal pass: lane = output row, warp w = outputs 4w .. 4w+3 of
        // it, from mid columns 8w .. 8w+17
        float b[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
        for (int j = 0; j < 18; ++j) {
            const float v = mid[lane][8 * warp + j];
#pragma unroll
            for (int r = 0; r < 4; ++r)
                if (j - 2 * r >= 0 && j - 2 * r < kLz2xTaps) b[r] = __fadd_rn(b[r], __fmul_rn(v, uni.wh[j - 2 * r]));
        }
        const long long od = (long long)(oy0 + lane) * dst_pitch + ox0 + 4 * warp;
        unsigned packed = 0u;
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            const float t = b[r] < 0.0f ? 0.0f : (b[r] > 255.0f ? 255.0f : b[r]);
            const int v = (int)roundf(t);
            store_level(dst + od + r, v, norm255(v));
            packed |= (unsigned)v << (8 * r);
        }
        *reinterpret_cast<unsigned*>(dst_u8 + od) = packed;
        return;
    }
    // vertical pass: rows oy0..oy1-1 (one warp per row), columns x_lo..x_hi-1
    for (int oyl = warp; oyl < oy1 - oy0; oyl += 8) {
        const int oy = oy0 + oyl;
        const int l = vleft[oy] - y_lo, c = vcount[oy], o = voff[oy];
        for (int xx = lane; xx < sw; xx += 32) {
            float t = 0.0f;
            for (int i = 0; i < c; ++i) t = __fadd_rn(t, __fmul_rn(in(l + i, xx), vw[o + i]));
            mid[oyl][xx] = t;
        }
    }
    __syncthreads();
    // horizontal pass
    for (int q = tid; q < (oy1 - oy0) * kLzT; q += 256) {
        const int oyl = q >> 5, oxl = q & 31;
        const int ox = ox0 + oxl;
        if (ox >= ox1) continue;
        const int l = hleft[ox] - x_lo, c = hcount[ox], o = hoff[ox];
        float t = 0.0f;
        for (int i = 0; i < c; ++i) t = __fadd_rn(t, __fmul_rn(mid[oyl][l + i], hw[o + i]));
        t = t < 0.0f ? 0.0f : (t > 255.0f ? 255.0f : t);
        const int v = (int)roundf(t);
        const long long od = (long long)(oy0 + oyl) * dst_pitch + ox;
        store_level(dst + od, v, norm255(v));
        dst_u8[od] = (uint8_t)v;
    }
}

template <typename TG>
__global__ void __launch_bounds__(256) k_lanczos_fused(const uint8_t* __restrict__ src, int src_pitch,
                                                       TG* __restrict__ dst, uint8_t* __restrict__ dst_u8,
                                                       int dst_pitch, int nW, int nH, const int* __restrict__ vtab,
                                                       const float* __restrict__ vw, const int* __restrict__ htab,
                                                       const float* __restrict__ hw, const LanczosUniform uni) {
    chain_wait();
    lanczos_tile<TG>(src, src_pitch, dst, dst_u8, dst_pitch, nW, nH, vtab, vw, htab, hw, uni, blockIdx.x * kLzT,
                     blockIdx.y * kLzT);
}

// Lanczos3 vertical pass (image 0.25.6 vertical_sample): tmp[oy][x] =
// sum_i G[left+i][x] * w_i, accumulated from 0 in tap order, kept in f32.
// Used when a tile's source window would not fit the fused kernel.
__global__ void k_lanczos_v(const uint8_t* __restrict__ src, int src_pitch, float* __restrict__ dst, int dst_pitch,
                            int W, int nH, const int* __restrict__ left, const int* __restrict__ count,
                            const int* __restrict__ woff, const float* __restrict__ w) {
    chain_wait();
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int oy = blockIdx.y;
    if (x >= W || oy >= nH) return;
    const int l = left[oy], c = count[oy], o = woff[oy];
    float t = 0.0f;
    for (int i = 0; i < c; ++i)
        t = __fadd_rn(t, __fmul_rn(float_of_u8(src[(long long)(l + i) * src_pitch + x]), w[o + i]));
    dst[(long long)oy * dst_pitch + x] = t;
}

// Lanczos3 horizontal pass (image 0.25.6 horizontal_sample): clamp to
// [0, 255], round half away from zero, store as the next octave's base level.
template <typename TG>
__global__ void k_lanczos_h(const float* __restrict__ src, int src_pitch, TG* __restrict__ dst,
                            uint8_t* __restrict__ dst_u8, int dst_pitch, int nW, int nH, const int* __restrict__ left,
                            const int* __restrict__ count, const int* __restrict__ woff,
                            const float* __restrict__ w) {
    chain_wait();
    const int ox = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y;
    if (ox >= nW || y >= nH) return;
    const int l = left[ox], c = count[ox], o = woff[ox];
    const float* row = src + (long long)y * src_pitch;
    float t = 0.0f;
    for (int i = 0; i < c; ++i) t = __fadd_rn(t, __fmul_rn(row[l + i], w[o + i]));
    t = t < 0.0f ? 0.0f : (t > 255.0f ? 255.0f : t);
    const int v = (int)roundf(t);
    const long long od = (long long)y * dst_pitch + ox;
    store_level(dst + od, v, norm255(v));
    dst_u8[od] = (uint8_t)v;
}

// ---------------------------------------------------------------------------
// Flattened batch launches. The entries of a batch are image-major (entry =
// image * O + octave); one launch covers octave o of every image. CTA b
// serves the image k with pref[k] <= b < pref[k + 1], where pref is the
// launch's prefix over the images' tile (or row) counts, and tile b - pref[k]
// of that image; the tile bodies are the single-image kernels' own.
__device__ __forceinline__ int find_image(const uint32_t* __restrict__ pref, int n, uint32_t b) {
    int lo = 0, hi = n;
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (pref[mid] <= b) lo = mid; else hi = mid;
    }
    return lo;
}

// level s of octave o from level s - 1 (from the input image when s == 0)
__device__ __forceinline__ const uint8_t* level_src(const BatchPyr& bp, const OctaveDev& od, int k, int s,
                                                    int* pitch) {
    if (s == 0) {
        *pitch = bp.img_pitch[k];
        return reinterpret_cast<const uint8_t*>(bp.img_addr[k]);
    }
    *pitch = od.pitch;
    return bp.U + od.u_off + (long long)(s - 1) * od.plane;
}

template <int R>
__global__ void __launch_bounds__(kFThreads) kb_blur_level(BatchPyr bp, int o, int s, int n_img,
                                                           const uint32_t* __restrict__ pref,
                                                           const float* __restrict__ wts,
                                                           const float* __restrict__ lut255) {
    chain_wait();
    extern __shared__ __align__(16) float sm[];
    const int k = find_image(pref, n_img, blockIdx.x);
    const OctaveDev od = bp.ents[k * bp.O + o];
    const int t = (int)(blockIdx.x - pref[k]), tx = (od.W + kFTX - 1) / kFTX;
    int in_pitch = 0;
    const uint8_t* in = level_src(bp, od, k, s, &in_pitch);
    uint8_t* out = bp.U + od.u_off + (long long)s * od.plane;
    blur_level_tile<uint8_t, R>(in, in_pitch, out, out, od.pitch, od.W, od.H, wts, lut255, (t % tx) * kFTX,
                                (t / tx) * kFTY, sm);
}

__global__ void __launch_bounds__(kRowThreads) kb_blur_rows(BatchPyr bp, uint8_t* __restrict__ tmp, int o, int s,
                                                            int r, int n_img, const uint32_t* __restrict__ pref,
                                                            const float* __restrict__ wts) {
    chain_wait();
    extern __shared__ __align__(16) float sm[];
    const int k = find_image(pref, n_img, blockIdx.x);
    const OctaveDev od = bp.ents[k * bp.O + o];
    int in_pitch = 0;
    const uint8_t* in = level_src(bp, od, k, s, &in_pitch);
    blur_row(in, in_pitch, tmp + od.t_off, od.pitch, od.W, r, wts, (int)(blockIdx.x - pref[k]), sm);
}

__global__ void __launch_bounds__(kColThreads) kb_blur_cols(BatchPyr bp, const uint8_t* __restrict__ tmp, int o,
                                                            int s, int r, int n_img,
                                                            const uint32_t* __restrict__ pref,
                                                            const float* __restrict__ wts,
                                                            const float* __restrict__ lut255) {
    chain_wait();
    extern __shared__ __align__(16) float sm[];
    const int k = find_image(pref, n_img, blockIdx.x);
    const OctaveDev od = bp.ents[k * bp.O + o];
    const int t = (int)(blockIdx.x - pref[k]), tx = (od.W + kColTX - 1) / kColTX;
    uint8_t* out = bp.U + od.u_off + (long long)s * od.plane;
    blur_cols_tile<uint8_t>(tmp + od.t_off, od.pitch, out, out, od.pitch, od.W, od.H, r, wts, lut255,
                            (t % tx) * kColTX, (t / tx) * kColRows, sm);
}

// Lanczos tables of one image's resize from octave o to o + 1 (offsets into
// the batch's integer and weight tables).
struct BatchLz {
    int vtab, vw, htab, hw;
    LanczosUniform uni;
};

__global__ void __launch_bounds__(256) kb_lanczos(BatchPyr bp, int o, int n_img, const uint32_t* __restrict__ pref,
                                                  const BatchLz* __restrict__ lz, const int* __restrict__ itab,
                                                  const float* __restrict__ ftab) {
    chain_wait();
    const int k = find_image(pref, n_img, blockIdx.x);
    const int e = k * bp.O + o;
    const OctaveDev od = bp.ents[e], nx = bp.ents[e + 1];
    const BatchLz& z = lz[e];
    const int t = (int)(blockIdx.x - pref[k]), tx = (nx.W + kLzT - 1) / kLzT;
    uint8_t* dst = bp.U + nx.u_off;
    lanczos_tile<uint8_t>(bp.U + od.u_off + (long long)bp.S * od.plane, od.pitch, dst, dst, nx.pitch, nx.W, nx.H,
                          itab + z.vtab, ftab + z.vw, itab + z.htab, ftab + z.hw, z.uni, (t % tx) * kLzT,
                          (t / tx) * kLzT);
}

}  // namespace

// ---- launchers ----------------------------------------------------------------

size_t blur_rows_smem(int W, int r) {
    int taps = 2 * r + 1;
    return sizeof(float) * ((size_t)((taps + 3) & ~3) + (size_t)W + 2 * (size_t)r + 8);
}
size_t blur_cols_smem(int r) {
    return sizeof(float) * ((size_t)taps8(r) + 256 + (size_t)(kColRows + taps8(r) - 1) * kColTX);
}

static int set_smem(const void* k, size_t smem) {
    if (smem <= 48 * 1024) return 0;
    return cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) == cudaSuccess ? 0 : -1;
}

// One level from the previous level's u8 plane: fused when r <= 8 and r <=
// fused_max_radius (the horizontal pass recomputes a 2r-row halo per tile,
// which stops paying beyond r = 8), on tiles of tile_rows (64 or 32) rows,
// else the two separable passes.
template <typename TG, int TY>
using BlurLevelKernel = void (*)(const uint8_t*, int, TG*, uint8_t*, int, int, int, const float*, const float*,
                                 const ImgRef*);
template <typename TG, int TY>
BlurLevelKernel<TG, TY> blur_level_kernel(int r) {
    switch (r) {
        case 1: return k_blur_level<TG, 1, TY>;
        case 2: return k_blur_level<TG, 2, TY>;
        case 3: return k_blur_level<TG, 3, TY>;
        case 4: return k_blur_level<TG, 4, TY>;
        case 5: return k_blur_level<TG, 5, TY>;
        case 6: return k_blur_level<TG, 6, TY>;
        case 7: return k_blur_level<TG, 7, TY>;
        default: return k_blur_level<TG, 8, TY>;
    }
}

template <typename TG, int TY>
int launch_blur_level_fused(const uint8_t* in, int in_pitch, TG* out, uint8_t* out_u8, int pitch, int W, int H,
                            int r, const float* wts, const float* lut255, cudaStream_t st, const ImgRef* ref) {
    const BlurLevelKernel<TG, TY> kern = blur_level_kernel<TG, TY>(r);
    const size_t smem = blur_fused_smem(r, TY);
    if (set_smem((const void*)kern, smem)) return -1;
    dim3 grid((W + kFTX - 1) / kFTX, (H + TY - 1) / TY);
    if (launch_chained(kern, grid, 4 * TY, smem, st, in, in_pitch, out, out_u8, pitch, W, H, wts, lut255, ref) !=
        cudaSuccess)
        return -1;
    return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
}

template <typename TG>
int launch_blur_level(const uint8_t* in, int in_pitch, uint8_t* tmp, TG* out, uint8_t* out_u8, int pitch, int W,
                      int H, int r, const float* wts, const float* lut255, cudaStream_t st, int* launches,
                      int fused_max_radius, const ImgRef* ref, int tile_rows) {
    if (r <= kFMaxR && r <= fused_max_radius) {
        const int rc = tile_rows == 32
                           ? launch_blur_level_fused<TG, 32>(in, in_pitch, out, out_u8, pitch, W, H, r, wts, lut255,
                                                             st, ref)
                           : launch_blur_level_fused<TG, 64>(in, in_pitch, out, out_u8, pitch, W, H, r, wts, lut255,
                                                             st, ref);
        if (rc) return rc;
        *launches += 1;
        return 0;
    }
    const size_t rs = blur_rows_smem(W, r), cs = blur_cols_smem(r);
    if (set_smem((const void*)k_blur_rows, rs) || set_smem((const void*)k_blur_cols<TG>, cs)) return -1;
    if (launch_chained(k_blur_rows, H, kRowThreads, rs, st, in, in_pitch, tmp, pitch, W, r, wts, ref) !=
        cudaSuccess)
        return -1;
    dim3 grid((W + kColTX - 1) / kColTX, (H + kColRows - 1) / kColRows);
    if (launch_chained(k_blur_cols<TG>, grid, kColThreads, cs, st, tmp, pitch, out, out_u8, pitch, W, H, r, wts,
                       lut255) != cudaSuccess)
        return -1;
    *launches += 2;
    return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
}

template <typename TG>
int launch_copy_level(const TG* prev, const uint8_t* prev_u8, TG* out, uint8_t* out_u8, int pitch, int W,
                      int H, cudaStream_t st) {
    dim3 grid((W + 255) / 256, H);
    if (launch_chained(k_copy_level<TG>, grid, 256, 0, st, prev, prev_u8, out, out_u8, pitch, W, H) != cudaSuccess)
        return -1;
    return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
}

template <typename TG>
int launch_u8_to_level(const uint8_t* img, long long stride, TG* out, uint8_t* out_u8, int pitch, int W, int H,
                       cudaStream_t st, const ImgRef* ref) {
    dim3 grid((W + 255) / 256, H);
    if (launch_chained(k_u8_to_level<TG>, grid, 256, 0, st, img, stride, out, out_u8, pitch, W, H, ref) !=
        cudaSuccess)
        return -1;
    return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
}

template <typename TG>
int launch_lanczos(const uint8_t* src, int src_pitch, int W, int H, float* tmp, int tmp_pitch, TG* dst,
                   uint8_t* dst_u8, int dst_pitch, int nW, int nH, const int* vtab, const float* vw, const int* htab,
                   const float* hw, const LanczosUniform& uni, cudaStream_t st, bool fused, int* launches) {
    if (fused) {
        dim3 g((nW + kLzT - 1) / kLzT, (nH + kLzT - 1) / kLzT);
        if (launch_chained(k_lanczos_fused<TG>, g, 256, 0, st, src, src_pitch, dst, dst_u8, dst_pitch, nW, nH, vtab,
                           vw, htab, hw, uni) != cudaSuccess)
            return -1;
        *launches += 1;
        return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
    }
    dim3 gv((W + 127) / 128, nH);
    if (launch_chained(k_lanczos_v, gv, 128, 0, st, src, src_pitch, tmp, tmp_pitch, W, nH, vtab, vtab + nH,
                       vtab + 2 * nH, vw) != cudaSuccess)
        return -1;
    dim3 gh((nW + 127) / 128, nH);
    if (launch_chained(k_lanczos_h<TG>, gh, 128, 0, st, tmp, tmp_pitch, dst, dst_u8, dst_pitch, nW, nH, htab,
                       htab + nW, htab + 2 * nW, hw) != cudaSuccess)
        return -1;
    (void)H;
    *launches += 2;
    return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
}

int lanczos_fused_span() { return kLzSpan; }

// ---- flattened batch launchers ------------------------------------------------

int blur_level_tiles(int W, int H) { return W > 0 && H > 0 ? ((W + kFTX - 1) / kFTX) * ((H + kFTY - 1) / kFTY) : 0; }
int blur_col_tiles(int W, int H) {
    return W > 0 && H > 0 ? ((W + kColTX - 1) / kColTX) * ((H + kColRows - 1) / kColRows) : 0;
}
int lanczos_tiles(int nW, int nH) { return nW > 0 && nH > 0 ? ((nW + kLzT - 1) / kLzT) * ((nH + kLzT - 1) / kLzT) : 0; }
size_t batch_lz_bytes() { return sizeof(BatchLz); }
void batch_lz_fill(void* out, int vtab, int vw, int htab, int hw, const LanczosUniform& uni) {
    BatchLz z{vtab, vw, htab, hw, uni};
    std::memcpy(out, &z, sizeof z);
}

// Level s of octave o of every image of a batch: the fused kernel (r <= 8,
// tiles prefixed by fused_pref) or the two passes (rows prefixed by
// rows_pref, column tiles by cols_pref; tmp holds each entry's
// horizontal-pass plane at its t_off).
int launch_blur_level_flat(const BatchPyr& bp, uint8_t* tmp, int o, int s, int r, int n_img,
                           const uint32_t* fused_pref, uint32_t n_fused, const uint32_t* rows_pref, uint32_t n_rows,
                           int max_w, const uint32_t* cols_pref, uint32_t n_cols, const float* wts,
                           const float* lut255, cudaStream_t st, int* launches, int fused_max_radius) {
    if (r <= kFMaxR && r <= fused_max_radius) {
        if (n_fused == 0) return 0;
        void (*kern)(BatchPyr, int, int, int, const uint32_t*, const float*, const float*);
        switch (r) {
            case 1: kern = kb_blur_level<1>; break;
            case 2: kern = kb_blur_level<2>; break;
            case 3: kern = kb_blur_level<3>; break;
            case 4: kern = kb_blur_level<4>; break;
            case 5: kern = kb_blur_level<5>; break;
            case 6: kern = kb_blur_level<6>; break;
            case 7: kern = kb_blur_level<7>; break;
            default: kern = kb_blur_level<8>; break;
        }
        const size_t smem = blur_fused_smem(r);
        if (set_smem((const void*)kern, smem)) return -1;
        if (launch_chained(kern, n_fused, kFThreads, smem, st, bp, o, s, n_img, fused_pref, wts, lut255) !=
            cudaSuccess)
            return -1;
        *launches += 1;
        return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
    }
    if (n_rows == 0) return 0;
    const size_t rs = blur_rows_smem(max_w, r), cs = blur_cols_smem(r);
    if (set_smem((const void*)kb_blur_rows, rs) || set_smem((const void*)kb_blur_cols, cs)) return -1;
    if (launch_chained(kb_blur_rows, n_rows, kRowThreads, rs, st, bp, tmp, o, s, r, n_img, rows_pref, wts) !=
        cudaSuccess)
        return -1;
    if (launch_chained(kb_blur_cols, n_cols, kColThreads, cs, st, bp, (const uint8_t*)tmp, o, s, r, n_img, cols_pref,
                       wts, lut255) != cudaSuccess)
        return -1;
    *launches += 2;
    return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
}

// The 2x Lanczos3 resize of octave o to o + 1 of every image (every resize
// fits the fused kernel; the caller checks).
int launch_lanczos_flat(const BatchPyr& bp, int o, int n_img, const uint32_t* pref, uint32_t n_tiles,
                        const void* lz, const int* itab, const float* ftab, cudaStream_t st) {
    if (n_tiles == 0) return 0;
    if (launch_chained(kb_lanczos, n_tiles, 256, 0, st, bp, o, n_img, pref, (const BatchLz*)lz, itab, ftab) !=
        cudaSuccess)
        return -1;
    return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
}
int lanczos_fused_tile() { return kLzT; }

#define SIFT_INST(TG)                                                                                              \
    template int launch_blur_level<TG>(const uint8_t*, int, uint8_t*, TG*, uint8_t*, int, int, int, int,           \
                                       const float*, const float*, cudaStream_t, int*, int, const ImgRef*, int);   \
    template int launch_copy_level<TG>(const TG*, const uint8_t*, TG*, uint8_t*, int, int, int,                    \
                                       cudaStream_t);                                                              \
    template int launch_u8_to_level<TG>(const uint8_t*, long long, TG*, uint8_t*, int, int, int, cudaStream_t,     \
                                        const ImgRef*);                                                            \
    template int launch_lanczos<TG>(const uint8_t*, int, int, int, float*, int, TG*, uint8_t*, int, int, int,      \
                                    const int*, const float*, const int*, const float*, const LanczosUniform&,      \
                                    cudaStream_t, bool, int*);
SIFT_INST(float)
SIFT_INST(__half)
SIFT_INST(uint8_t)
#undef SIFT_INST

}  // namespace sift
