// detect.cu — 26-neighbour extrema, subpixel refinement, ordered compaction.
//
// Stages (b) and (c) of the hot path: find_scale_space_extrema
// (src/sift.rs:510-603) and refine_and_filter_extrema (src/sift.rs:299-474).
//
//   k_extrema_mask   one warp per 32 consecutive pixels of a row: the strict
//                    26-neighbour test, one ballot word per warp (no atomics).
//   scan             exclusive prefix sum of popcount(word) gives every
//                    candidate its slot in (octave, layer, y, x) order, the
//                    order rayon's collect produces in the reference.
//   k_emit           one thread per word writes the word's candidates to their
//                    slots.
//   k_refine         one thread per candidate: the Newton refinement, contrast
//                    and edge tests in the reference's f32 operation order;
//                    the result stays in the candidate's slot with a keep
//                    flag (the orientation stage reads the slots in order and
//                    skips the rejected ones, so no compaction pass is needed).
//
// All arithmetic is f32 with separately rounded operations (no FMA), so the
// candidates and refined keypoints are bit-identical to the CPU path; the one
// transcendental, 2^(octave + layer/S) for the keypoint size, is evaluated in
// f64 and rounded once.
#include <algorithm>

#include "sift_internal.cuh"

namespace sift {
namespace {

// DoG access for one octave (src/sift.rs:208-214 get_pixel_value, clamped).
// DoG of one octave recomputed from the u8 copies of its Gaussian levels:
// D_l = lut[G_{l+1}] - lut[G_l] with lut[v] = v/255 in f32 — the reference's
// f32 DoG bit for bit (src/sift.rs:92-124) in either storage mode, at one byte
// per level value instead of four (the refinement's scattered 3 x 3 x 3 reads
// then mostly hit L2).
struct DogFromU8 {
    const uint8_t* base;  // u8 level 0 of the octave
    const float* lut;     // v / 255, shared or global
    long long plane;
    int pitch, W, H;
    __device__ __forceinline__ float at(int l, int x, int y) const {
        x = clampi(x, 0, W - 1);
        y = clampi(y, 0, H - 1);
        const uint8_t* p = base + (long long)l * plane + (long long)y * pitch + x;
        return __fsub_rn(lut[p[plane]], lut[p[0]]);
    }
};

// DoG staged from the u8 copies of the Gaussian levels of one octave:
// D_l = lut[G_{l+1}] - lut[G_l] with lut[v] = v/255 in f32, which is the
// reference's f32 DoG bit for bit (src/sift.rs:92-124) at a quarter of the
// bytes.
// Stages layers 0..L-1 of the clamped window [x0, x0+TW) x [y0, y0+TH) into
// tile[L][TH][TW]; windows inside the plane go as aligned 4-byte words, all
// L+1 levels of a word per thread.
__device__ __forceinline__ void stage_dog_u8(float* tile, const float* lut, const uint8_t* base, long long plane,
                                             int pitch, int W, int H, int L, int x0, int y0, int TW, int TH, int tid,
                                             int nthreads) {
    const bool inner = x0 >= 0 && y0 >= 0 && x0 + TW <= W && y0 + TH <= H && (x0 & 3) == 0 && (TW & 3) == 0 &&
                       (pitch & 3) == 0;
    if (inner) {
        const int q4 = TW >> 2;
        for (int q = tid; q < TH * q4; q += nthreads) {
            const int yy = q / q4, xx = (q - yy * q4) * 4;
            const uint8_t* p = base + (long long)(y0 + yy) * pitch + x0 + xx;
            const unsigned b0 = *reinterpret_cast<const unsigned*>(p);
            float lo0 = lut[b0 & 0xffu], lo1 = lut[(b0 >> 8) & 0xffu], lo2 = lut[(b0 >> 16) & 0xffu],
                  lo3 = lut[b0 >> 24];
            float* t = tile + yy * TW + xx;
#pragma unroll 4
            for (int l = 0; l < L; ++l) {
                const unsigned b = *reinterpret_cast<const unsigned*>(p + (long long)(l + 1) * plane);
                const float u0 = lut[b & 0xffu], u1 = lut[(b >> 8) & 0xffu], u2 = lut[(b >> 16) & 0xffu],
                            u3 = lut[b >> 24];
                *reinterpret_cast<float4*>(t + (size_t)l * TH * TW) =
                    make_float4(__fsub_rn(u0, lo0), __fsub_rn(u1, lo1), __fsub_rn(u2, lo2), __fsub_rn(u3, lo3));
                lo0 = u0;
                lo1 = u1;
                lo2 = u2;
                lo3 = u3;
            }
        }
    } else {
        for (int q = tid; q < TH * TW; q += nthreads) {
            const int yy = q / TW, xx = q - yy * TW;
            const long long o = (long long)clampi(y0 + yy, 0, H - 1) * pitch + clampi(x0 + xx, 0, W - 1);
            float lo = lut[base[o]];
            for (int l = 0; l < L; ++l) {
                const float up = lut[base[(long long)(l + 1) * plane + o]];
                tile[(l * TH + yy) * TW + xx] = __fsub_rn(up, lo);
                lo = up;
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Extrema of one octave, all layers s = 1..S at once. The CTA stages the
// neighbourhood of its 64 x 16 pixels for every DoG layer 0..S+1 in shared
// memory, formed from the u8 levels (clamped coordinates, as get_pixel_value
// clamps, at the image border). Each thread owns one column and 4 rows: per
// layer it forms the horizontal 3-max/3-min of 6 rows once and reuses them for
// the 3x3 block max/min and the 8-ring max/min of its 4 pixels:
//   strict max  <=>  v > max(M_{s-1}, M_{s+1}, ring8max_s)
//   strict min  <=>  v < min(m_{s-1}, m_{s+1}, ring8min_s)
// which is the reference's 26 strict comparisons (ties reject).
constexpr int kExTX = 64, kExTY = 16, kExRows = 4, kExMaxLayers = 18;
constexpr int kExSW = kExTX + 8;  // staged width: x0-4 .. x0+68 (word aligned)
constexpr int kExSH = kExTY + 2;

// NL > 0: the number of DoG layers (S + 2) is compiled in and the layer loop
// unrolls, so the sliding window renames registers instead of moving them;
// NL == 0: any S.
template <int NL>
__device__ __forceinline__ void extrema_tile(const uint8_t* __restrict__ u8arena, const float* __restrict__ lut255,
                                             const OctaveDev& od, int S, int border, uint32_t* __restrict__ words,
                                             int x0, int y0, float* tile) {
    const int W = od.W, H = od.H, nw = od.nw, L = NL > 0 ? NL : S + 2;
    const int tid = threadIdx.x, lane = tid & 31;
    float* lut = tile + L * kExSH * kExSW;
    lut[tid] = lut255[tid];
    __syncthreads();
    stage_dog_u8(tile, lut, u8arena + od.u_off, od.plane, od.pitch, W, H, L, x0 - 4, y0 - 1, kExSW, kExSH, tid, 256);
    __syncthreads();
    const int col = tid & (kExTX - 1);          // 0..63
    const int r0 = (tid >> 6) * kExRows;       // 0, 4, 8, 12
    const int x = x0 + col;
    const int tx = col + 4;                     // staged column of x
    const int word = (x0 >> 5) + ((tid >> 5) & 1);  // this warp's 32 columns
    const bool xin = x >= border && x < W - border;
    bool yin[kExRows];
#pragma unroll
    for (int j = 0; j < kExRows; ++j) yin[j] = xin && y0 + r0 + j >= border && y0 + r0 + j < H - border;
    // Sliding window over the layers: p = l-2, c = l-1, n = l.
    float BMp[kExRows], Bmp[kExRows], BMc[kExRows], Bmc[kExRows], RMc[kExRows], Rmc[kExRows], Vc[kExRows];
#pragma unroll
    for (int j = 0; j < kExRows; ++j) BMp[j] = Bmp[j] = BMc[j] = Bmc[j] = RMc[j] = Rmc[j] = Vc[j] = 0.0f;
#pragma unroll
    for (int l = 0; l < (NL > 0 ? NL : L); ++l) {
        const float* t = tile + (l * kExSH + r0) * kExSW + tx;  // staged row y0 + r0 - 1
        float left[kExRows + 2], mid[kExRows + 2], right[kExRows + 2], hM[kExRows + 2], hm[kExRows + 2];
#pragma unroll
        for (int j = 0; j < kExRows + 2; ++j) {
            left[j] = t[j * kExSW - 1];
            mid[j] = t[j * kExSW];
            right[j] = t[j * kExSW + 1];
            hM[j] = fmaxf(fmaxf(left[j], mid[j]), right[j]);
            hm[j] = fminf(fminf(left[j], mid[j]), right[j]);
        }
        float BMn[kExRows], Bmn[kExRows], RMn[kExRows], Rmn[kExRows];
#pragma unroll
        for (int j = 0; j < kExRows; ++j) {
            BMn[j] = fmaxf(fmaxf(hM[j], hM[j + 1]), hM[j + 2]);
            Bmn[j] = fminf(fminf(hm[j], hm[j + 1]), hm[j + 2]);
            RMn[j] = fmaxf(fmaxf(hM[j], hM[j + 2]), fmaxf(left[j + 1], right[j + 1]));
            Rmn[j] = fminf(fminf(hm[j], hm[j + 2]), fminf(left[j + 1], right[j + 1]));
        }
        if (l >= 2) {
            const int s = l - 1;  // centre layer
#pragma unroll
            for (int j = 0; j < kExRows; ++j) {
                const int y = y0 + r0 + j;
                const float v = Vc[j];
                const bool ext = yin[j] && ((v > fmaxf(fmaxf(BMp[j], BMn[j]), RMc[j])) ||
                                            (v < fminf(fminf(Bmp[j], Bmn[j]), Rmc[j])));
                const uint32_t wv = __ballot_sync(0xffffffffu, ext);
                if (lane == 0 && y < H && word < nw) words[od.word_base + ((long long)(s - 1) * H + y) * nw + word] = wv;
            }
        }
#pragma unroll
        for (int j = 0; j < kExRows; ++j) {
            BMp[j] = BMc[j];
            Bmp[j] = Bmc[j];
            BMc[j] = BMn[j];
            Bmc[j] = Bmn[j];
            RMc[j] = RMn[j];
            Rmc[j] = Rmn[j];
            Vc[j] = mid[j + 1];
        }
    }
}

// The extrema mask of entry e (one octave of one image), a tile per CTA.
template <int NL>
__global__ void __launch_bounds__(256, 4) k_extrema_mask(const uint8_t* __restrict__ u8arena,
                                                      const float* __restrict__ lut255, EntryTable tab, int e,
                                                      int border, uint32_t* __restrict__ words) {
    chain_wait();
    extern __shared__ __align__(16) float tile[];  // [layers][kExSH][kExSW], then lut[256]
    const OctaveDev od = tab.ents[e];
    extrema_tile<NL>(u8arena, lut255, od, tab.S, border, words, blockIdx.x * kExTX, blockIdx.y * kExTY, tile);
}

// The extrema masks of entries e0 .. e0 + n_e - 1 in one launch: CTA b takes
// tile b - tile_pref[k] of entry e0 + k, tile_pref[k] <= b < tile_pref[k + 1]
// (row-major tiles of kExTX x kExTY).
template <int NL>
__global__ void __launch_bounds__(256, 4) k_extrema_mask_flat(const uint8_t* __restrict__ u8arena,
                                                           const float* __restrict__ lut255, EntryTable tab, int e0,
                                                           int n_e, const uint32_t* __restrict__ tile_pref,
                                                           int border, uint32_t* __restrict__ words) {
    chain_wait();
    extern __shared__ __align__(16) float tile[];
    const uint32_t b = blockIdx.x;
    int lo = 0, hi = n_e;  // the last k with tile_pref[k] <= b
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (tile_pref[mid] <= b) lo = mid; else hi = mid;
    }
    const OctaveDev od = tab.ents[e0 + lo];
    const int tx = (od.W + kExTX - 1) / kExTX;
    const int t = (int)(b - tile_pref[lo]);
    extrema_tile<NL>(u8arena, lut255, od, tab.S, border, words, (t % tx) * kExTX, (t / tx) * kExTY, tile);
}

// solve_linear_system (src/sift.rs:478-503), Cramer's rule in f32.
__device__ __forceinline__ bool solve3(const float a[3][3], const float b[3], float x[3]) {
#define M(p, q) __fmul_rn(p, q)
#define S(p, q) __fsub_rn(p, q)
#define A(p, q) __fadd_rn(p, q)
    const float det_a = A(S(M(a[0][0], S(M(a[1][1], a[2][2]), M(a[1][2], a[2][1]))),
                            M(a[0][1], S(M(a[1][0], a[2][2]), M(a[1][2], a[2][0])))),
                          M(a[0][2], S(M(a[1][0], a[2][1]), M(a[1][1], a[2][0]))));
    if (fabsf(det_a) < 1e-10f) return false;
    const float det_x = A(S(M(b[0], S(M(a[1][1], a[2][2]), M(a[1][2], a[2][1]))),
                            M(a[0][1], S(M(b[1], a[2][2]), M(a[1][2], b[2])))),
                          M(a[0][2], S(M(b[1], a[2][1]), M(a[1][1], b[2]))));
    const float det_y = A(S(M(a[0][0], S(M(b[1], a[2][2]), M(a[1][2], b[2]))),
                            M(b[0], S(M(a[1][0], a[2][2]), M(a[1][2], a[2][0])))),
                          M(a[0][2], S(M(a[1][0], b[2]), M(b[1], a[2][0]))));
    const float det_z = A(S(M(a[0][0], S(M(a[1][1], b[2]), M(b[1], a[2][1]))),
                            M(a[0][1], S(M(a[1][0], b[2]), M(b[1], a[2][0])))),
                          M(b[0], S(M(a[1][0], a[2][1]), M(a[1][1], a[2][0]))));
#undef M
#undef S
#undef A
    x[0] = __fdiv_rn(det_x, det_a);
    x[1] = __fdiv_rn(det_y, det_a);
    x[2] = __fdiv_rn(det_z, det_a);
    return true;
}

struct RefineParams {
    float sigma;
    float contrast_threshold;
    float edge_threshold;
    int S;
    int levels_dog;  // S + 2
};

// One candidate through refine_and_filter_extrema (src/sift.rs:299-474).
template <class Dog>
__device__ bool refine_one(const Dog& dog, int o, int entry, int x, int y, int s, const RefineParams& rp,
                           Keypoint* out) {
    int cx = x, cy = y, cl = s;
    const float scale = __int_as_float((127 + o) << 23);  // 2^o
    const int nl = rp.levels_dog;
    for (int step = 0; step < 5; ++step) {
        if (cl < 1 || cl >= nl - 1) return false;
        if (cx < 1 || cx >= dog.W - 1 || cy < 1 || cy >= dog.H - 1) return false;
        const int lp = cl - 1, lc = cl, ln = cl + 1;
        const float c = dog.at(lc, cx, cy);
        const float cxp = dog.at(lc, cx + 1, cy), cxm = dog.at(lc, cx - 1, cy);
        const float cyp = dog.at(lc, cx, cy + 1), cym = dog.at(lc, cx, cy - 1);
        const float nc = dog.at(ln, cx, cy), pc = dog.at(lp, cx, cy);
        const float dx = __fdiv_rn(__fsub_rn(cxp, cxm), 2.0f);
        const float dy = __fdiv_rn(__fsub_rn(cyp, cym), 2.0f);
        const float ds = __fdiv_rn(__fsub_rn(nc, pc), 2.0f);
        const float c2 = __fmul_rn(2.0f, c);
        const float dxx = __fsub_rn(__fadd_rn(cxp, cxm), c2);
        const float dyy = __fsub_rn(__fadd_rn(cyp, cym), c2);
        const float dss = __fsub_rn(__fadd_rn(nc, pc), c2);
        const float dxy = __fdiv_rn(__fadd_rn(__fsub_rn(__fsub_rn(dog.at(lc, cx + 1, cy + 1), dog.at(lc, cx - 1, cy + 1)),
                                                        dog.at(lc, cx + 1, cy - 1)),
                                              dog.at(lc, cx - 1, cy - 1)),
                                    4.0f);
        const float dxs = __fdiv_rn(__fsub_rn(__fsub_rn(dog.at(ln, cx + 1, cy), dog.at(ln, cx - 1, cy)),
                                              __fsub_rn(dog.at(lp, cx + 1, cy), dog.at(lp, cx - 1, cy))),
                                    4.0f);
        const float dys = __fdiv_rn(__fsub_rn(__fsub_rn(dog.at(ln, cx, cy + 1), dog.at(ln, cx, cy - 1)),
                                              __fsub_rn(dog.at(lp, cx, cy + 1), dog.at(lp, cx, cy - 1))),
                                    4.0f);
        const float hm[3][3] = {{dxx, dxy, dxs}, {dxy, dyy, dys}, {dxs, dys, dss}};
        const float g[3] = {-dx, -dy, -ds};
        float off[3];
        if (!solve3(hm, g, off)) return false;
        if (fabsf(off[0]) < 0.5f && fabsf(off[1]) < 0.5f && fabsf(off[2]) < 0.5f) {
            const float lin = __fadd_rn(__fadd_rn(__fmul_rn(dx, off[0]), __fmul_rn(dy, off[1])), __fmul_rn(ds, off[2]));
            const float val = __fadd_rn(c, __fmul_rn(0.5f, lin));
            if (fabsf(val) < rp.contrast_threshold) return false;
            const float tr = __fadd_rn(dxx, dyy);
            const float trace_sq = __fmul_rn(tr, tr);
            const float det = __fsub_rn(__fmul_rn(dxx, dyy), __fmul_rn(dxy, dxy));
            if (det <= 0.0f) return false;
            const float ratio = __fdiv_rn(trace_sq, det);
            const float e1 = __fadd_rn(rp.edge_threshold, 1.0f);
            const float thr = __fdiv_rn(__fmul_rn(e1, e1), rp.edge_threshold);
            if (ratio >= thr) return false;
            const float lf = __fadd_rn((float)cl, off[2]);
            const float e = __fadd_rn((float)o, __fdiv_rn(lf, (float)rp.S));
            const float p2 = (float)exp2((double)e);
            out->x = __fmul_rn(__fadd_rn((float)cx, off[0]), scale);
            out->y = __fmul_rn(__fadd_rn((float)cy, off[1]), scale);
            out->size = __fmul_rn(rp.sigma, p2);
            out->angle = 0.0f;
            out->response = val;
            out->octave = entry;
            out->layer = rust_as_i32(roundf(lf));
            return true;
        }
        cx = rust_as_i32(roundf(__fadd_rn((float)cx, off[0])));
        cy = rust_as_i32(roundf(__fadd_rn((float)cy, off[1])));
        cl = rust_as_i32(roundf(__fadd_rn((float)cl, off[2])));
        if (cl < 0 || cl >= nl) return false;
    }
    return false;
}

// One thread per mask word of entries e0 .. e0 + n_e - 1 (their words are
// consecutive; w counts from the first entry's first word): the candidates of
// the word go to their scanned slots, in x order within the word, i.e.
// (entry, layer, y, x) order. A candidate's octave field holds its entry.
__global__ void __launch_bounds__(256) k_emit(const uint8_t* __restrict__ u8arena, const float* __restrict__ lut255,
                                              EntryTable tab, int e0, int n_e, long long n_words,
                                              const uint32_t* __restrict__ words,
                                              const uint32_t* __restrict__ cand_off,
                                              Keypoint* __restrict__ cands, uint32_t cap,
                                              Counters* __restrict__ ctr) {
    chain_wait();
    const long long w = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= n_words) return;
    uint32_t word = words[w];
    if (word == 0u) return;
    const long long base0 = tab.ents[e0].word_base;
    int lo = 0, hi = n_e;  // the last entry whose first word is <= w
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (tab.ents[e0 + mid].word_base - base0 <= w) lo = mid; else hi = mid;
    }
    const int e = e0 + lo;
    const OctaveDev od = tab.ents[e];
    const long long we = w - (od.word_base - base0);
    const DogFromU8 dog{u8arena + od.u_off, lut255, od.plane, od.pitch, od.W, od.H};
    const int c = (int)(we % od.nw);
    const long long rowid = we / od.nw;
    const int y = (int)(rowid % od.H);
    const int s = (int)(rowid / od.H) + 1;
    const float scale = __int_as_float((127 + od.octave) << 23);
    uint32_t ci = cand_off[w];
    while (word) {
        const int b = __ffs(word) - 1;
        word &= word - 1u;
        const int x = c * 32 + b;
        if (ci >= cap) {
            atomicOr(&ctr->overflow, 1u);
            return;
        }
        Keypoint k;
        k.x = __fmul_rn(__fadd_rn((float)x, 0.5f), scale);
        k.y = __fmul_rn(__fadd_rn((float)y, 0.5f), scale);
        k.size = 0.0f;
        k.angle = 0.0f;
        k.response = dog.at(s, x, y);
        k.octave = e;
        k.layer = s;
        cands[ci++] = k;
    }
}

// One thread per candidate (persistent grid over the count); a candidate's
// entry (its octave field) gives its octave and DoG planes. The survivors are
// counted per warp into oc->n_ref (a count, order-free).
__global__ void __launch_bounds__(256) k_refine(const uint8_t* __restrict__ u8arena,
                                                const float* __restrict__ lut255, EntryTable tab,
                                                RefineParams rp, const Keypoint* __restrict__ cands,
                                                Keypoint* __restrict__ refined_at, uint32_t* __restrict__ keep,
                                                uint32_t cap, OctCounters* __restrict__ oc) {
    chain_wait();
    __shared__ float lut[256];
    lut[threadIdx.x] = lut255[threadIdx.x];
    __syncthreads();
    const uint32_t n = min(oc->n_cand, cap);
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t i0 = blockIdx.x * blockDim.x; i0 < n; i0 += stride) {
        const uint32_t i = i0 + threadIdx.x;
        bool ok = false;
        if (i < n) {
            const Keypoint k = cands[i];
            const OctaveDev od = tab.ents[k.octave];
            const DogFromU8 dog{u8arena + od.u_off, lut, od.plane, od.pitch, od.W, od.H};
            const float scale = __int_as_float((127 + od.octave) << 23);
            const int x = rust_as_i32(__fdiv_rn(k.x, scale)), y = rust_as_i32(__fdiv_rn(k.y, scale));
            Keypoint r;
            ok = refine_one(dog, od.octave, k.octave, x, y, k.layer, rp, &r);
            if (ok) refined_at[i] = r;
            keep[i] = ok ? 1u : 0u;
        }
        const uint32_t m = __ballot_sync(0xffffffffu, ok);
        if ((threadIdx.x & 31) == 0 && m) atomicAdd(&oc->n_ref, (uint32_t)__popc(m));
    }
}

// Debug read-back of DoG layer l of octave o as a dense W x H f32 plane, each
// value formed by DogFromU8::at, the function the candidate emission and the
// refinement read DoG through (u8 planes and the v / 255 table in device
// memory). Not part of a run.
__global__ void k_dog_dense(const uint8_t* __restrict__ u8arena, const float* __restrict__ lut255, PyramidDev pyr,
                            int o, int l, float* __restrict__ out) {
    chain_wait();
    const OctaveDev& od = pyr.oct[o];
    const DogFromU8 dog{u8arena + od.u_off, lut255, od.plane, od.pitch, od.W, od.H};
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
    if (x < od.W && y < od.H) out[(long long)y * od.W + x] = dog.at(l, x, y);
}

}  // namespace

// ---- launchers -------------------------------------------------------------

int launch_dog_dense(const uint8_t* u8arena, const float* lut255, const PyramidDev& pyr, int o, int l, float* out,
                     cudaStream_t st) {
    const OctaveDev& od = pyr.oct[o];
    if (od.W <= 0 || od.H <= 0) return 0;
    dim3 grid((od.W + 127) / 128, od.H);
    if (launch_chained(k_dog_dense, grid, 128, 0, st, u8arena, lut255, pyr, o, l, out) != cudaSuccess) return -1;
    return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
}

static size_t extrema_smem(int S) { return sizeof(float) * ((size_t)(S + 2) * kExSH * kExSW + 256); }

int launch_extrema_mask(const uint8_t* u8arena, const float* lut255, const EntryTable& tab, const OctaveDev& od,
                        int e, int border, uint32_t* words, cudaStream_t st) {
    if (od.W <= 0 || od.H <= 0) return 0;
    if (tab.S + 2 > kExMaxLayers) return -1;
    dim3 grid((od.W + kExTX - 1) / kExTX, (od.H + kExTY - 1) / kExTY);
    const size_t smem = extrema_smem(tab.S);
    void (*k)(const uint8_t*, const float*, EntryTable, int, int, uint32_t*) =
        tab.S == 3 ? k_extrema_mask<5> : (tab.S == 4 ? k_extrema_mask<6> : k_extrema_mask<0>);
    if (smem > 48 * 1024 &&
        cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return -1;
    if (launch_chained(k, grid, 256, smem, st, u8arena, lut255, tab, e, border, words) != cudaSuccess)
        return -1;
    return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
}

int extrema_tiles(int W, int H) {
    return W > 0 && H > 0 ? ((W + kExTX - 1) / kExTX) * ((H + kExTY - 1) / kExTY) : 0;
}

int launch_extrema_mask_flat(const uint8_t* u8arena, const float* lut255, const EntryTable& tab, int e0, int n_e,
                             const uint32_t* tile_pref, uint32_t n_tiles, int border, uint32_t* words,
                             cudaStream_t st) {
    if (n_tiles == 0) return 0;
    if (tab.S + 2 > kExMaxLayers) return -1;
    const size_t smem = extrema_smem(tab.S);
    void (*k)(const uint8_t*, const float*, EntryTable, int, int, const uint32_t*, int, uint32_t*) =
        tab.S == 3 ? k_extrema_mask_flat<5> : (tab.S == 4 ? k_extrema_mask_flat<6> : k_extrema_mask_flat<0>);
    if (smem > 48 * 1024 &&
        cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return -1;
    if (launch_chained(k, n_tiles, 256, smem, st, u8arena, lut255, tab, e0, n_e, tile_pref, border, words) !=
        cudaSuccess)
        return -1;
    return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
}

int launch_emit(const uint8_t* u8arena, const float* lut255, const EntryTable& tab, int e0, int n_e,
                long long n_words, const uint32_t* words, const uint32_t* cand_off, Keypoint* cands, uint32_t cap,
                Counters* ctr, cudaStream_t st) {
    if (n_words <= 0) return 0;
    unsigned grid = (unsigned)((n_words + 255) / 256);
    if (launch_chained(k_emit, grid, 256, 0, st, u8arena, lut255, tab, e0, n_e, n_words, words, cand_off, cands, cap,
                       ctr) != cudaSuccess)
        return -1;
    return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
}

// Refinement is a chain of dependent scattered reads per candidate: up to
// 5 CTAs of 8 warps per SM keep enough of them in flight.
int launch_refine(const uint8_t* u8arena, const float* lut255, const EntryTable& tab, float sigma, float contrast,
                  float edge, const Keypoint* cands, Keypoint* refined_at, uint32_t* keep, uint32_t cap,
                  OctCounters* oc, cudaStream_t st) {
    RefineParams rp{sigma, contrast, edge, tab.S, tab.S + 2};
    const unsigned grid = (unsigned)std::min<size_t>(((size_t)cap + 255) / 256, 152 * 5);
    if (launch_chained(k_refine, grid, 256, 0, st, u8arena, lut255, tab, rp, cands, refined_at, keep, cap, oc) !=
        cudaSuccess)
        return -1;
    return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace sift
