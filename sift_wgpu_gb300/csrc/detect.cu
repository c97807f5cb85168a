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
//   k_emit_refine    re-reads the words; each candidate lane writes its
//                    candidate record and runs the Newton refinement, contrast
//                    and edge tests in the reference's f32 operation order.
//                    Survivors are aggregated per warp with a ballot.
//   scan + k_compact survivors move to their final slots, order kept.
//
// All arithmetic is f32 with separately rounded operations (no FMA), so the
// candidates and refined keypoints are bit-identical to the CPU path; the one
// transcendental, 2^(octave + layer/S) for the keypoint size, is evaluated in
// f64 and rounded once.
#include "sift_internal.cuh"

namespace sift {
namespace {

// DoG access for one octave (src/sift.rs:208-214 get_pixel_value, clamped).
struct DogF32 {
    const float* base;  // DoG level 0 of the octave
    long long plane;
    int pitch, W, H;
    __device__ __forceinline__ float at(int l, int x, int y) const {
        x = clampi(x, 0, W - 1);
        y = clampi(y, 0, H - 1);
        return base[(long long)l * plane + (long long)y * pitch + x];
    }
};

// DoG recomputed in f32 from f16-stored Gaussian levels:
// D_l = G_{l+1}/255 - G_l/255, exactly as stored DoG would hold it.
struct DogFromG16 {
    const __half* base;  // G level 0 of the octave
    long long plane;
    int pitch, W, H;
    __device__ __forceinline__ float at(int l, int x, int y) const {
        x = clampi(x, 0, W - 1);
        y = clampi(y, 0, H - 1);
        const long long o = (long long)y * pitch + x;
        float a = __half2float(base[(long long)(l + 1) * plane + o]);
        float b = __half2float(base[(long long)l * plane + o]);
        return __fsub_rn(__fdiv_rn(a, 255.0f), __fdiv_rn(b, 255.0f));
    }
};

template <class Dog>
__device__ __forceinline__ Dog make_dog(const void* arena, const OctaveDev& od);
template <>
__device__ __forceinline__ DogF32 make_dog<DogF32>(const void* arena, const OctaveDev& od) {
    return DogF32{(const float*)arena + od.d_off, od.plane, od.pitch, od.W, od.H};
}
template <>
__device__ __forceinline__ DogFromG16 make_dog<DogFromG16>(const void* arena, const OctaveDev& od) {
    return DogFromG16{(const __half*)arena + od.g_off, od.plane, od.pitch, od.W, od.H};
}

// ---------------------------------------------------------------------------
template <class Dog>
__global__ void __launch_bounds__(256) k_extrema_mask(const void* arena, PyramidDev pyr, int o, int border,
                                                      uint32_t* __restrict__ words) {
    const OctaveDev& od = pyr.oct[o];
    const Dog dog = make_dog<Dog>(arena, od);
    const int W = od.W, H = od.H, nw = od.nw;
    const int lane = threadIdx.x;
    const int c = blockIdx.x;
    const int y = blockIdx.y * 8 + threadIdx.y;
    const int s = blockIdx.z + 1;
    const int x = c * 32 + lane;
    bool ext = false;
    if (y >= border && y < H - border && x >= border && x < W - border) {
        const float v = dog.at(s, x, y);
        bool is_max = true, is_min = true;
#pragma unroll
        for (int dz = -1; dz <= 1; ++dz)
#pragma unroll
            for (int dy = -1; dy <= 1; ++dy)
#pragma unroll
                for (int dx = -1; dx <= 1; ++dx) {
                    if (dz == 0 && dy == 0 && dx == 0) continue;
                    const float n = dog.at(s + dz, x + dx, y + dy);
                    is_max = is_max && (v > n);
                    is_min = is_min && (v < n);
                }
        ext = is_max || is_min;
    }
    const uint32_t m = __ballot_sync(0xffffffffu, ext);
    if (lane == 0 && y < H) words[od.word_base + ((long long)(s - 1) * H + y) * nw + c] = m;
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
__device__ bool refine_one(const Dog& dog, int o, int x, int y, int s, const RefineParams& rp, Keypoint* out) {
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
            out->octave = o;
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

__device__ __forceinline__ int find_octave(const PyramidDev& pyr, long long w) {
    int o = 0;
    for (int k = 1; k < pyr.num_octaves; ++k)
        if (pyr.oct[k].word_base <= w) o = k;
    return o;
}

template <class Dog>
__global__ void __launch_bounds__(256) k_emit_refine(const void* arena, PyramidDev pyr, long long n_words,
                                                     const uint32_t* __restrict__ words,
                                                     const uint32_t* __restrict__ cand_off, RefineParams rp,
                                                     Keypoint* __restrict__ cands, Keypoint* __restrict__ refined_at,
                                                     uint32_t* __restrict__ keep_mask,
                                                     uint32_t* __restrict__ keep_count, uint32_t cap,
                                                     Counters* __restrict__ ctr) {
    const long long w = (long long)blockIdx.x * 8 + threadIdx.y;
    if (w >= n_words) return;  // whole warp exits together
    const int lane = threadIdx.x;
    const uint32_t word = words[w];
    if (word == 0u) {
        if (lane == 0) {
            keep_mask[w] = 0u;
            keep_count[w] = 0u;
        }
        return;
    }
    const int o = find_octave(pyr, w);
    const OctaveDev& od = pyr.oct[o];
    const long long local = w - od.word_base;
    const int c = (int)(local % od.nw);
    const long long rowid = local / od.nw;
    const int y = (int)(rowid % od.H);
    const int s = (int)(rowid / od.H) + 1;
    const int x = c * 32 + lane;
    const bool is_cand = (word >> lane) & 1u;
    bool keep = false;
    if (is_cand) {
        const uint32_t ci = cand_off[w] + (uint32_t)__popc(word & ((1u << lane) - 1u));
        const Dog dog = make_dog<Dog>(arena, od);
        if (ci < cap) {
            const float scale = __int_as_float((127 + o) << 23);
            Keypoint k;
            k.x = __fmul_rn(__fadd_rn((float)x, 0.5f), scale);
            k.y = __fmul_rn(__fadd_rn((float)y, 0.5f), scale);
            k.size = 0.0f;
            k.angle = 0.0f;
            k.response = dog.at(s, x, y);
            k.octave = o;
            k.layer = s;
            cands[ci] = k;
            Keypoint r;
            keep = refine_one(dog, o, x, y, s, rp, &r);
            if (keep) refined_at[ci] = r;
        } else {
            atomicOr(&ctr->overflow, 1u);
        }
    }
    const uint32_t km = __ballot_sync(0xffffffffu, keep);
    if (lane == 0) {
        keep_mask[w] = km;
        keep_count[w] = (uint32_t)__popc(km);
    }
}

__global__ void __launch_bounds__(256) k_compact(long long n_words, const uint32_t* __restrict__ words,
                                                 const uint32_t* __restrict__ cand_off,
                                                 const uint32_t* __restrict__ keep_mask,
                                                 const uint32_t* __restrict__ keep_off,
                                                 const Keypoint* __restrict__ refined_at,
                                                 Keypoint* __restrict__ refined, uint32_t cap) {
    const long long w = (long long)blockIdx.x * 8 + threadIdx.y;
    if (w >= n_words) return;
    const uint32_t km = keep_mask[w];
    if (km == 0u) return;
    const int lane = threadIdx.x;
    if (!((km >> lane) & 1u)) return;
    const uint32_t lt = (1u << lane) - 1u;
    const uint32_t ci = cand_off[w] + (uint32_t)__popc(words[w] & lt);
    const uint32_t ri = keep_off[w] + (uint32_t)__popc(km & lt);
    if (ci < cap && ri < cap) refined[ri] = refined_at[ci];
}

}  // namespace

// ---- launchers -------------------------------------------------------------

int launch_extrema_mask(int storage, const void* arena, const PyramidDev& pyr, int o, int border, uint32_t* words,
                        cudaStream_t st) {
    const OctaveDev& od = pyr.oct[o];
    if (od.W <= 0 || od.H <= 0) return 0;
    dim3 grid(od.nw, (od.H + 7) / 8, pyr.S);
    if (storage == SIFT_CUDA_STORAGE_F16)
        k_extrema_mask<DogFromG16><<<grid, dim3(32, 8), 0, st>>>(arena, pyr, o, border, words);
    else
        k_extrema_mask<DogF32><<<grid, dim3(32, 8), 0, st>>>(arena, pyr, o, border, words);
    return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
}

int launch_emit_refine(int storage, const void* arena, const PyramidDev& pyr, long long n_words,
                       const uint32_t* words, const uint32_t* cand_off, float sigma, float contrast, float edge,
                       Keypoint* cands, Keypoint* refined_at, uint32_t* keep_mask, uint32_t* keep_count,
                       uint32_t cap, Counters* ctr, cudaStream_t st) {
    if (n_words <= 0) return 0;
    RefineParams rp{sigma, contrast, edge, pyr.S, pyr.S + 2};
    unsigned grid = (unsigned)((n_words + 7) / 8);
    if (storage == SIFT_CUDA_STORAGE_F16)
        k_emit_refine<DogFromG16><<<grid, dim3(32, 8), 0, st>>>(arena, pyr, n_words, words, cand_off, rp, cands,
                                                                refined_at, keep_mask, keep_count, cap, ctr);
    else
        k_emit_refine<DogF32><<<grid, dim3(32, 8), 0, st>>>(arena, pyr, n_words, words, cand_off, rp, cands,
                                                            refined_at, keep_mask, keep_count, cap, ctr);
    return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
}

int launch_compact(long long n_words, const uint32_t* words, const uint32_t* cand_off, const uint32_t* keep_mask,
                   const uint32_t* keep_off, const Keypoint* refined_at, Keypoint* refined, uint32_t cap,
                   cudaStream_t st) {
    if (n_words <= 0) return 0;
    unsigned grid = (unsigned)((n_words + 7) / 8);
    k_compact<<<grid, dim3(32, 8), 0, st>>>(n_words, words, cand_off, keep_mask, keep_off, refined_at, refined, cap);
    return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace sift
