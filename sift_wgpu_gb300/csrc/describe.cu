// describe.cu — orientation assignment and 4x4x8 descriptors (sm_103a).
//
// Stages (d) and (e) of the hot path: assign_orientations
// (src/sift.rs:605-726) and compute (src/sift.rs:917-1060) with
// normalize_and_clip_descriptor (src/sift.rs:889-913).
//
//   k_orientation   one warp per refined keypoint (orient_one): the (2r+1)^2
//                   window is split over the lanes, each lane takes its samples
//                   two at a time and adds them into its own column of a
//                   bin-major shared histogram (conflict-free, no atomics),
//                   columns are summed in a fixed order, then the two [1,1,1]/3
//                   smoothing passes and the peak test run one bin per lane;
//                   peaks come out in bin order through a ballot.
//   k_orient_emit   candidate slot i with c_i peaks (0 if refinement rejected
//                   it) writes its c_i oriented copies at the scanned offset,
//                   so the output order is the reference's (keypoint, bin)
//                   order.
//   k_descriptor    one CTA per oriented keypoint (describe_one): the bilinear
//                   samples of the window are computed once into a shared grid,
//                   pairs of window samples are split over the threads and
//                   evaluated on packed f32x2 arithmetic, trilinear
//                   contributions are added into 128 shared bins as u32 fixed
//                   point (integer addition is associative, so the result does
//                   not depend on scheduling), then L2 normalise, clip at 0.2,
//                   renormalise.
// Both queues run from the last item of an octave's list (the largest
// windows first).
//
// The orientation histogram follows the reference's f32 operation order
// without FMA, except the Gaussian weight (hardware exponential of a
// reciprocal product) and the angle (polynomial atan2 away from bin edges,
// atan2f and the IEEE division next to them, so every bin index is exact);
// its column sums are in a fixed order. The descriptor loop trades exactness
// for speed within the descriptor tolerance (see describe_one). Orientations
// and descriptors therefore agree with the reference within rounding, not bit
// for bit.
#include <algorithm>
#include <type_traits>

#include "sift_internal.cuh"

namespace sift {
namespace {

constexpr int kOriWarps = 8;  // orientation: one keypoint per warp

// Work-queue kernels launch more CTAs than fit on the device. A CTA (or an
// orientation warp) below persist_from takes at most kBudget items and
// retires, which frees its slot for kernels of more urgent streams (the
// smaller octaves' chains) instead of holding it until the queue drains; the
// CTAs from persist_from on, the last wave, loop until the queue is empty,
// so every item is taken whatever the grid.
constexpr int kOriBudget = 4;   // keypoints per warp
constexpr int kDescBudget = 2;  // keypoints per CTA

// A Gaussian level pixel as v/255 (get_gauss_pixel_value, src/sift.rs:218-223):
// f32 levels store it directly, f16 and u8 levels store v, divided here
// (div255 is the IEEE quotient for every u8 value), so every storage mode
// reads the same values.
template <typename T>
__device__ __forceinline__ float gnorm(const T* p);
template <>
__device__ __forceinline__ float gnorm<float>(const float* p) {
    return *p;
}
template <>
__device__ __forceinline__ float gnorm<__half>(const __half* p) {
    return div255(__half2float(*p));
}
template <>
__device__ __forceinline__ float gnorm<uint8_t>(const uint8_t* p) {
    return div255(float_of_u8(*p));
}

// The same pixel as v itself (0..255): f32 levels give it back exactly as
// fl(fl(v / 255) * 255) (true for every u8 value), f16 and u8 levels store it.
// The descriptor works in these units: its histogram is L2-normalised, so the
// factor 255 cancels, and the three storage modes give the same values.
template <typename T>
__device__ __forceinline__ float graw(const T* p);
template <>
__device__ __forceinline__ float graw<float>(const float* p) {
    return __fmul_rn(*p, 255.0f);
}
template <>
__device__ __forceinline__ float graw<__half>(const __half* p) {
    return __half2float(*p);
}
template <>
__device__ __forceinline__ float graw<uint8_t>(const uint8_t* p) {
    return float_of_u8(*p);
}

template <typename TG>
struct GaussPlane {
    const TG* base;
    int pitch, W, H;
    // u8 levels: v / 255 from this table (shared memory) when given, else
    // by div255; both are the IEEE quotient
    const float* lut;
    __device__ __forceinline__ float at(const TG* p) const {
        if constexpr (std::is_same<TG, uint8_t>::value) {
            if (lut) return lut[*p];
        }
        return gnorm(p);
    }
    // get_gauss_pixel_value (src/sift.rs:218-223)
    __device__ __forceinline__ float px(int x, int y) const {
        x = clampi(x, 0, W - 1);
        y = clampi(y, 0, H - 1);
        return at(base + (long long)y * pitch + x);
    }
    // the same for coordinates already inside the level
    __device__ __forceinline__ float px_in(int x, int y) const { return at(base + y * pitch + x); }
    // get_gauss_pixel_value in v units (graw)
    __device__ __forceinline__ float px_raw(int x, int y) const {
        x = clampi(x, 0, W - 1);
        y = clampi(y, 0, H - 1);
        return graw(base + (long long)y * pitch + x);
    }
    // get_gauss_pixel_bilinear (src/sift.rs:238-266)
    __device__ __forceinline__ float bilinear(float x, float y) const {
        const float xf = floorf(x), yf = floorf(y);
        const float xc = __fadd_rn(xf, 1.0f), yc = __fadd_rn(yf, 1.0f);
        const float dx = __fsub_rn(x, xf), dy = __fsub_rn(y, yf);
        const int x0 = rust_as_i32(xf), y0 = rust_as_i32(yf), x1 = rust_as_i32(xc), y1 = rust_as_i32(yc);
        const float q11 = px(x0, y0), q21 = px(x1, y0), q12 = px(x0, y1), q22 = px(x1, y1);
        const float omx = __fsub_rn(1.0f, dx), omy = __fsub_rn(1.0f, dy);
        float v = __fmul_rn(__fmul_rn(q11, omx), omy);
        v = __fadd_rn(v, __fmul_rn(__fmul_rn(q21, dx), omy));
        v = __fadd_rn(v, __fmul_rn(__fmul_rn(q12, omx), dy));
        v = __fadd_rn(v, __fmul_rn(__fmul_rn(q22, dx), dy));
        return v;
    }
};

template <typename TG>
__device__ __forceinline__ GaussPlane<TG> plane_for(const TG* arena, const OctaveDev& od, int S, int layer,
                                                    const float* lut = nullptr) {
    const int li = clampi(layer, 0, S + 2);
    return GaussPlane<TG>{arena + od.g_off + (long long)li * od.plane, od.pitch, od.W, od.H, lut};
}


// The exact orientation bin position of a gradient angle (src/sift.rs:652-656):
// atan2 in (-pi, pi] to [0, 2 pi), times 36, divided by 2 pi.
__device__ __forceinline__ float exact_bin_pos(float ang) {
    const float two_pi = 2.0f * kPi;
    const float an = ang < 0.0f ? __fadd_rn(ang, two_pi) : ang;
    return __fdiv_rn(__fmul_rn(an, (float)kOriBins), two_pi);  // in [0, 36]
}

// Bin positions of the four axis directions. The levels are quantised, so
// many gradients have gx or gy exactly 0; their angles (0, pi/2, pi, -pi/2)
// fall exactly on bin edges, where only the exact sequence decides the bin.
// They are computed once with that sequence instead of per sample.
struct AxisBins {
    float right, up, left, down;  // angle 0, pi/2, pi, -pi/2
};
__device__ __forceinline__ AxisBins axis_bins() {
    return AxisBins{exact_bin_pos(atan2f(0.0f, 1.0f)), exact_bin_pos(atan2f(1.0f, 0.0f)),
                    exact_bin_pos(atan2f(0.0f, -1.0f)), exact_bin_pos(atan2f(-1.0f, 0.0f))};
}

// One orientation sample (src/sift.rs:640-662) into the lane's column of the
// bin-major histogram hist[bin][32]: the gradient (gx, gy) at window offset
// (fdx, fdy), added as +0.0 when the sample lies outside the level (`in`
// false), which leaves a bin bit-identical.
// bf: the polynomial bin position of the gradient (ori_bin_pos2).
__device__ __forceinline__ void ori_add(float gx, float gy, float fdx, float fdy, float inv_wd, bool in,
                                        float* hist, int lane, const AxisBins& ab, float bf) {
    // the hardware square root (within an ulp; the bins are sums whose
    // order differs from the reference's anyway)
    const float mag = sqrt_approx(__fadd_rn(__fmul_rn(gx, gx), __fmul_rn(gy, gy)));
    // exp(-(dx^2 + dy^2) / wd) with the quotient as a product by 1 / wd and
    // the hardware exponential: a few ulp from expf of the IEEE quotient,
    // the same order as expf's own distance from the host libm
    const float wgt = __expf(__fmul_rn(-__fadd_rn(__fmul_rn(fdx, fdx), __fmul_rn(fdy, fdy)), inv_wd));
    // Bin index: from the polynomial atan2 and a multiply by 36 / (2 pi)
    // (a few ulp from the exact value); axis directions take their exact
    // position from the table; any other angle within 1e-4 of a bin edge
    // takes atan2f and the IEEE division, the exact sequence (rare: the
    // branch no longer splits warps on every flat patch). Away from the
    // edges all three floor to the same bin.
    const bool axis = gx == 0.0f || gy == 0.0f;  // (0, 0): atan2 0, angle 0
    const float bax = gy == 0.0f ? (gx < 0.0f ? ab.left : ab.right) : (gy > 0.0f ? ab.up : ab.down);
    bf = axis ? bax : bf;
    if (!axis && fabsf(__fsub_rn(bf, rintf(bf))) < 1e-4f) bf = exact_bin_pos(atan2f(gy, gx));
    const int fl = floor_i(bf);
    const int bin = fl >= kOriBins ? fl - kOriBins : fl;
    const float v = __fmul_rn(mag, wgt);
    float* h = hist + bin * 32 + lane;
    *h = __fadd_rn(*h, in ? v : 0.0f);
}

// The polynomial bin positions of two gradients: atan2_poly to [0, 2 pi),
// times 36 / (2 pi) (src/sift.rs:652-656), on f32x2 pairs.
__device__ __forceinline__ float2 ori_bin_pos2(float2 gy, float2 gx) {
    const float two_pi = 2.0f * kPi;
    const float2 pa = atan2_poly2(gy, gx);
    const float2 pw = __fadd2_rn(pa, make_float2(two_pi, two_pi));
    const float2 pn = make_float2(pa.x < 0.0f ? pw.x : pa.x, pa.y < 0.0f ? pw.y : pa.y);
    const float k = (float)kOriBins / two_pi;
    return __fmul2_rn(pn, make_float2(k, k));
}

// The orientation window of one keypoint (src/sift.rs:640-662), lane-strided:
// sample k = lane + 32 j of the (2r+1)^2 window, read from the level (the
// reads mostly hit L1). A lane takes its samples two at a time (k and
// k + 32: their loads in flight together, the two arctangents on f32x2
// pairs) and adds them to its histogram column in window order, as one at a
// time would. Windows at the level's border take the CHECK form.
template <typename TG, bool CHECK>
__device__ __forceinline__ void ori_window(const GaussPlane<TG>& g, float xo, float yo, int r, float wd, float* hist,
                                           int lane, const AxisBins& ab) {
    const float inv_wd = __frcp_rn(wd);
    const int side = 2 * r + 1;
    const float side_f = (float)side, r_f = (float)r;
    // Sample k = lane + 32 j of the window (row-major) is (fdx, fdy) =
    // (k % side - r, k / side - r): exact small integers in f32 that advance
    // by fixed amounts per step, with one row wrap (as selects) at most.
    const int q0 = lane / side, dq = 32 / side;
    const float dr_f = (float)(32 - dq * side), dq_f = (float)dq;
    auto wrap = [&](float& x, float& y) {
        const bool w = x > r_f;
        x = w ? x - side_f : x;
        y = w ? y + 1.0f : y;
    };
    // the gradient at a window offset (src/sift.rs:640-651)
    auto grad = [&](float fdx, float fdy, float& gx, float& gy, bool& in) {
        int xi = round_away_i(__fadd_rn(xo, fdx));
        int yi = round_away_i(__fadd_rn(yo, fdy));
        in = true;
        if (CHECK) {
            in = !(xi < 1 || xi >= g.W - 1 || yi < 1 || yi >= g.H - 1);
            xi = clampi(xi, 1, g.W - 2);
            yi = clampi(yi, 1, g.H - 2);
        }
        gx = __fsub_rn(g.px_in(xi + 1, yi), g.px_in(xi - 1, yi));
        gy = __fsub_rn(g.px_in(xi, yi + 1), g.px_in(xi, yi - 1));
    };
    float fdx = (float)(lane - q0 * side) - r_f, fdy = (float)q0 - r_f;
    for (;;) {
        wrap(fdx, fdy);
        if (fdy > r_f) break;
        float fdx1 = fdx + dr_f, fdy1 = fdy + dq_f;
        wrap(fdx1, fdy1);
        const bool has1 = fdy1 <= r_f;  // else the second reads the first's offset and is not added
        float gx0, gy0, gx1, gy1;
        bool in0, in1;
        grad(fdx, fdy, gx0, gy0, in0);
        grad(has1 ? fdx1 : fdx, has1 ? fdy1 : fdy, gx1, gy1, in1);
        const float2 bf = ori_bin_pos2(make_float2(gy0, gy1), make_float2(gx0, gx1));
        ori_add(gx0, gy0, fdx, fdy, inv_wd, in0, hist, lane, ab, bf.x);
        if (has1) ori_add(gx1, gy1, fdx1, fdy1, inv_wd, in1, hist, lane, ab, bf.y);
        fdx = fdx1 + dr_f;
        fdy = fdy1 + dq_f;
    }
}

// The orientation peaks of one refined keypoint (src/sift.rs:605-726),
// computed by one warp: the window into the warp's bin-major histogram
// hist[36][32], the column sums and the two smoothing passes in hs[36], the
// peaks in bin order written to angles[0 .. count). Returns the count (the
// same in every lane).
template <typename TG>
__device__ __forceinline__ uint32_t orient_one(const TG* __restrict__ arena, const EntryTable& tab, const Keypoint& kp,
                                               float* hist, float* hs, int lane, const AxisBins& ab,
                                               float* __restrict__ angles, const float* lut) {
    const float two_pi = 2.0f * kPi;
    const float bin_w = 2.0f * kPi / (float)kOriBins;
    const int e = kp.octave;  // entry
    if (!(e >= 0 && e < tab.n)) return 0;
    const OctaveDev od = tab.ents[e];
    const int o = od.octave;
    const GaussPlane<TG> g = plane_for(arena, od, tab.S, kp.layer, lut);
    const float scale = __int_as_float((127 + o) << 23);
    const float xo = __fdiv_rn(kp.x, scale), yo = __fdiv_rn(kp.y, scale);
    const float so = __fdiv_rn(kp.size, scale);
    if (!(so > 0.0f)) return 0;
    const int r = rust_as_i32(roundf(__fmul_rn(4.5f, so)));
    const float ws = __fmul_rn(1.5f, so);
    const float wd = __fmul_rn(__fmul_rn(2.0f, ws), ws);
#pragma unroll
    for (int b = 0; b < kOriBins; ++b) hist[b * 32 + lane] = 0.0f;

    // Windows entirely inside the level (most keypoints) take the loop
    // without bounds checks; the others add +0.0 for samples outside, which
    // leaves a bin bit-identical.
    const bool interior = xo - (float)r >= 2.5f && xo + (float)r <= (float)(g.W - 3) - 0.5f &&
                          yo - (float)r >= 2.5f && yo + (float)r <= (float)(g.H - 3) - 0.5f;
    if (interior)
        ori_window<TG, false>(g, xo, yo, r, wd, hist, lane, ab);
    else
        ori_window<TG, true>(g, xo, yo, r, wd, hist, lane, ab);
    __syncwarp();
    // Column sums: bin `lane` in four interleaved partial sums (the column
    // index rotated by the bin keeps the 32 lanes in 32 banks), bins 32..35
    // by eight lanes each and a shuffle tree.
    {
        const float* hb = hist + lane * 32;
        float s0 = 0.0f, s1 = 0.0f, s2 = 0.0f, s3 = 0.0f;
#pragma unroll
        for (int l = 0; l < 32; l += 4) {
            s0 = __fadd_rn(s0, hb[(l + lane) & 31]);
            s1 = __fadd_rn(s1, hb[(l + 1 + lane) & 31]);
            s2 = __fadd_rn(s2, hb[(l + 2 + lane) & 31]);
            s3 = __fadd_rn(s3, hb[(l + 3 + lane) & 31]);
        }
        hs[lane] = __fadd_rn(__fadd_rn(s0, s1), __fadd_rn(s2, s3));
        const int bb = 32 + (lane >> 3), c0 = (lane & 7) * 4;
        const float* ht = hist + bb * 32;
        float t = __fadd_rn(__fadd_rn(ht[(c0 + bb) & 31], ht[(c0 + 1 + bb) & 31]),
                            __fadd_rn(ht[(c0 + 2 + bb) & 31], ht[(c0 + 3 + bb) & 31]));
        t = __fadd_rn(t, __shfl_xor_sync(0xffffffffu, t, 1));
        t = __fadd_rn(t, __shfl_xor_sync(0xffffffffu, t, 2));
        t = __fadd_rn(t, __shfl_xor_sync(0xffffffffu, t, 4));
        if ((lane & 7) == 0) hs[bb] = t;
    }
    __syncwarp();
    for (int it = 0; it < 2; ++it) {
        float nv0 = 0.0f, nv1 = 0.0f;
        for (int b = lane, q = 0; b < kOriBins; b += 32, ++q) {
            const float v = __fdiv_rn(
                __fadd_rn(__fadd_rn(hs[(b + kOriBins - 1) % kOriBins], hs[b]), hs[(b + 1) % kOriBins]), 3.0f);
            if (q == 0) nv0 = v; else nv1 = v;
        }
        __syncwarp();
        for (int b = lane, q = 0; b < kOriBins; b += 32, ++q) hs[b] = q == 0 ? nv0 : nv1;
        __syncwarp();
    }
    float mx = fmaxf(hs[lane], lane + 32 < kOriBins ? hs[lane + 32] : 0.0f);
#pragma unroll
    for (int m = 16; m > 0; m >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, m));
    const float thr = __fmul_rn(mx, 0.8f);
    bool pk[2] = {false, false};
    float pa[2] = {0.0f, 0.0f};
    for (int b = lane, q = 0; b < kOriBins; b += 32, ++q) {
        const float cv = hs[b];
        if (!(cv >= thr)) continue;
        const float pv = hs[(b + kOriBins - 1) % kOriBins];
        const float nv = hs[(b + 1) % kOriBins];
        if (cv > pv && cv > nv) {
            const float den = __fadd_rn(__fsub_rn(pv, __fmul_rn(2.0f, cv)), nv);
            const float off = fabsf(den) > 1e-5f ? __fdiv_rn(__fmul_rn(0.5f, __fsub_rn(pv, nv)), den) : 0.0f;
            const float center = __fmul_rn(__fadd_rn((float)b, 0.5f), bin_w);
            const float a = __fadd_rn(center, __fmul_rn(off, bin_w));
            float fa = rem_euclid_2b(a, two_pi);  // a in (0, 2 pi + pi/36)
            if (fa > kPi) fa = __fsub_rn(fa, two_pi);
            pk[q] = true;
            pa[q] = fa;
        }
    }
    const uint32_t m0 = __ballot_sync(0xffffffffu, pk[0]);
    const uint32_t m1 = __ballot_sync(0xffffffffu, pk[1]);
    const uint32_t lt = (1u << lane) - 1u;
    if (pk[0]) angles[__popc(m0 & lt)] = pa[0];
    if (pk[1]) angles[__popc(m0) + __popc(m1 & lt)] = pa[1];
    __syncwarp();
    return (uint32_t)(__popc(m0) + __popc(m1));
}

template <typename TG>
__global__ void __launch_bounds__(32 * kOriWarps, 5) k_orientation(const TG* __restrict__ arena, EntryTable tab,
                                                                const float* __restrict__ lut255,
                                                                const Keypoint* __restrict__ refined_at,
                                                                const uint32_t* __restrict__ keep, uint32_t ncap,
                                                                OctCounters* __restrict__ oc,
                                                                float* __restrict__ ori_angle,
                                                                uint32_t* __restrict__ ori_count,
                                                                int persist_from) {
    chain_wait();
    __shared__ float hist[kOriWarps][kOriBins][32];
    __shared__ float hs[kOriWarps][kOriBins];
    // u8 levels: v / 255 from a shared copy of the table (one load per
    // pixel instead of a conversion and the three-instruction quotient)
    __shared__ float slut[256];
    const int lane = threadIdx.x, wid = threadIdx.y;
    constexpr bool kU8 = std::is_same<TG, uint8_t>::value;
    if (kU8) {
        for (int v = wid * 32 + lane; v < 256; v += 32 * kOriWarps) slut[v] = lut255[v];
        __syncthreads();
    }
    const uint32_t n = min(oc->n_cand, ncap);  // candidate slots; rejected ones get 0 peaks
    const AxisBins ab = axis_bins();
    const bool persist = (int)blockIdx.x >= persist_from;
    for (int taken = 0; persist || taken < kOriBudget; ++taken) {
        uint32_t i = 0;
        if (lane == 0) i = atomicAdd(&oc->next_ori, 1u);
        i = __shfl_sync(0xffffffffu, i, 0);
        if (i >= n) break;
        i = n - 1 - i;  // from the last slot: the largest windows first
        uint32_t cnt = 0;
        if (keep[i])
            cnt = orient_one<TG>(arena, tab, refined_at[i], &hist[wid][0][0], &hs[wid][0], lane, ab,
                                 ori_angle + (size_t)i * kOriMaxPeaks, kU8 ? slut : nullptr);
        if (lane == 0) ori_count[i] = cnt;
    }
}

// Octave o's oriented keypoints go after those of octaves 0..o-1 (whose
// counts are final: their orientation scans precede this kernel). Candidate
// slot i holds ori_count[i] peaks (0 for a rejected candidate).
__global__ void k_orient_emit(const Keypoint* __restrict__ refined_at, uint32_t ncap, int o,
                              Counters* __restrict__ ctr, const float* __restrict__ ori_angle,
                              const uint32_t* __restrict__ ori_count, const uint32_t* __restrict__ ori_off,
                              Keypoint* __restrict__ oriented, uint32_t cap) {
    chain_wait();
    OctCounters* oc = &ctr->oct[o];
    uint32_t base = 0;
    for (int q = 0; q < o; ++q) base += ctr->oct[q].n_ori;
    const uint32_t n = min(oc->n_cand, ncap);
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        oc->out_base = base;
        atomicAdd(&ctr->n_candidates, oc->n_cand);
        atomicAdd(&ctr->n_refined, oc->n_ref);
        atomicMax(&ctr->n_oriented, base + oc->n_ori);
        if (base + oc->n_ori > cap) atomicOr(&ctr->overflow, 4u);
    }
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t c = ori_count[i], off = base + ori_off[i];
        if (c == 0) continue;
        Keypoint k = refined_at[i];
        for (uint32_t j = 0; j < c; ++j) {
            if (off + j >= cap) break;
            k.angle = ori_angle[(size_t)i * kOriMaxPeaks + j];
            oriented[off + j] = k;
        }
    }
}

constexpr int kDescThreads = 128;
static_assert(kDescThreads == kDescLen && kDescThreads == 128, "one descriptor bin per thread, four warps");
constexpr int kHistRow = 9;      // 8 angle bins + slot 8, the share of bin 0 that wrapped from bin 7
constexpr int kHistSide = 6;     // cells -1..4 per axis: the 4 x 4 window and a border that takes the
                                 // trilinear spill, so no sample needs a clamp or a validity test
constexpr int kHistCopies = 8;   // lane & 7 picks the copy
constexpr int kHistStride = 324; // 36 * kHistRow; 324 % 32 = 4 puts a bin's 8 copies in 8 banks
constexpr int kDescRadGrid = 31;                      // largest radius served from the grid
constexpr int kDescGridSide = 2 * kDescRadGrid + 3;   // offsets -(rad+1) .. rad+1

// The descriptor of one oriented keypoint (src/sift.rs:917-1060 and
// normalize_and_clip_descriptor, src/sift.rs:889-913), computed by the whole
// CTA (kDescThreads threads; it synchronises the CTA) into dst[0 .. 128):
//  1. The bilinear samples the gradients need, bilinear(xo + i, yo + j) for
//     integer offsets i, j in [-(rad+1), rad+1], go to a shared grid once
//     (the reference re-evaluates four bilinears per window sample).
//  2. Each thread takes pairs of neighbouring window samples and evaluates
//     both at once with Blackwell's packed f32x2 multiply/add/FMA (the kernel
//     is bound by instruction issue); the eight trilinear contributions of
//     each are added to 128 shared bins as u32 fixed point (2^-f units, f
//     chosen so no bin can overflow): integer addition is associative, so the
//     descriptor is the same on every run.
//  3. The four warps normalise, clip at 0.2, renormalise.
// Radii above the grid (not reachable with the default sigma) fall back to
// per-sample bilinears from the level itself.
template <typename TG>
__device__ __forceinline__ void describe_one(const TG* __restrict__ arena, const EntryTable& tab, const Keypoint& kp,
                                             float* grid, unsigned int* hist, float* red_lo, float* red_hi,
                                             float* __restrict__ dst) {
    const int tid = threadIdx.x;
    const float sqrt2 = __fsqrt_rn(2.0f);
    const int e = kp.octave;  // entry
    for (int w = tid; w < kHistCopies * kHistStride / 4; w += kDescThreads)
        reinterpret_cast<uint4*>(hist)[w] = make_uint4(0u, 0u, 0u, 0u);
    const bool valid_oct = e >= 0 && e < tab.n;
    OctaveDev od{};
    if (valid_oct) od = tab.ents[e];
    const int o = od.octave;
    // division by 2^o is the multiplication by 2^-o, exactly
    const float inv_scale = valid_oct ? __int_as_float((127 - o) << 23) : 1.0f;
    const float so = valid_oct ? __fmul_rn(kp.size, inv_scale) : 0.0f;
    const bool valid = valid_oct && so > 0.0f;
    float inv_fix = 0.0f;
    if (valid) {
        const GaussPlane<TG> g = plane_for(arena, od, tab.S, kp.layer);
        const float xo = __fmul_rn(kp.x, inv_scale), yo = __fmul_rn(kp.y, inv_scale);
        const float ang = kp.angle;
        // the hardware sine and cosine (|ang| <= pi; absolute error ~4e-7,
        // a shift of ~1e-5 px at the window's edge)
        float sa, ca;
        __sincosf(ang, &sa, &ca);
        const float bw = __fmul_rn(3.0f, so);
        const float ww = __fmul_rn(bw, 4.0f);
        const float wsig = __fmul_rn(0.5f, ww);
        const float wd = __fmul_rn(__fmul_rn(2.0f, wsig), wsig);
        const int rad = rust_as_i32(ceilf(__fmul_rn(__fmul_rn(ww, sqrt2), 0.5f)));
        const float wm1 = (float)(g.W - 1), hm1 = (float)(g.H - 1);
        const int side = 2 * rad + 1;
        const int total = side * side;
        const bool use_grid = rad <= kDescRadGrid;
        const int gs = side + 2;
        // Grid layout: row gr (0 .. gs - 1) at gr * gst + (gr & 1), row
        // stride gst = gs + 1 (even), one spare slot per row (the last of
        // an even row, the first of an odd row). With the pair loop's
        // phase (the pairs of odd rows start one sample to the left), all
        // four float pairs a pair of samples reads are 8-byte aligned.
        const int gst = gs + 1;
        float lo = 3.0e38f, hi = 0.0f;
        if (use_grid) {
            // the spare slots, read only for the phantom element of a
            // row's end pair, hold 0
            if (tid < gs) grid[tid * gst + ((tid & 1) ? 0 : gs)] = 0.0f;
            // Bilinear samples at the window's integer offsets, in v units
            // (graw), straight from the level (the patch stays in L1). All
            // of them share the
            // fraction of (xo, yo): the reference's sample positions xo + i
            // differ from it only by the rounding of that sum. Clamped
            // reads (get_gauss_pixel_value) only for windows at the border.
            const float xf = floorf(xo), yf = floorf(yo);
            const float fdx = xo - xf, fdy = yo - yf;
            const int px0 = (int)xf - (rad + 1), py0 = (int)yf - (rad + 1);
            const bool inner = px0 >= 0 && py0 >= 0 && px0 + gs < g.W && py0 + gs < g.H;
            const float inv_gs = 1.0f / (float)gs;
            if (inner) {
                // A thread makes a strip of 4 x 2 grid points from 5 x 3
                // pixels: each row's horizontal lerps serve the points
                // above and below it, both columns at once on f32x2
                // pairs (15 loads for 8 points); consecutive lanes take
                // consecutive column pairs. The same two lerps per point
                // as below, so the same values.
                const int strips = (gs + 3) >> 2, cps = (gs + 1) >> 1;
                const float inv_cps = 1.0f / (float)cps;
                const TG* org = g.base + py0 * g.pitch + px0;
                const float2 fdx2 = make_float2(fdx, fdx), fdy2 = make_float2(fdy, fdy);
                const float2 neg1 = make_float2(-1.0f, -1.0f);
                float tf = (float)tid;
                for (int t = tid; t < strips * cps; t += kDescThreads, tf += (float)kDescThreads) {
                    const int sy = floor_i((tf + 0.5f) * inv_cps);
                    const int qx = 2 * (t - sy * cps), qy0 = 4 * sy;
                    const int nr = min(4, gs - qy0);
                    // an odd-width grid's last pair has a phantom second
                    // column: its third pixel repeats the second (in
                    // bounds) and nothing is stored for it
                    const bool two = qx + 1 < gs;
                    const int o2 = two ? 2 : 1;
                    // all 15 loads first (rows past the strip's last
                    // repeat it), then the lerps
                    const TG* pp = org + qy0 * g.pitch + qx;
                    float a[5][3];
#pragma unroll
                    for (int j = 0; j < 5; ++j) {
                        const TG* pr = pp + min(j, nr) * g.pitch;
                        a[j][0] = graw(pr);
                        a[j][1] = graw(pr + 1);
                        a[j][2] = graw(pr + o2);
                    }
                    float2 A = make_float2(a[0][0], a[0][1]);
                    float2 rp = __ffma2_rn(fdx2, __ffma2_rn(A, neg1, make_float2(a[0][1], a[0][2])), A);
                    float* gp = grid + qy0 * gst + qx;  // qy0 even
#pragma unroll
                    for (int j = 0; j < 4; ++j) {
                        A = make_float2(a[j + 1][0], a[j + 1][1]);
                        const float2 rn =
                            __ffma2_rn(fdx2, __ffma2_rn(A, neg1, make_float2(a[j + 1][1], a[j + 1][2])), A);
                        const float2 b = __ffma2_rn(fdy2, __ffma2_rn(rp, neg1, rn), rp);
                        if (j < nr) {
                            gp[j * gst + (j & 1)] = b.x;
                            if (two) gp[j * gst + (j & 1) + 1] = b.y;
                            lo = fminf(lo, fminf(b.x, b.y));
                            hi = fmaxf(hi, fmaxf(b.x, b.y));
                        }
                        rp = rn;
                    }
                }
            } else {
                float qf = (float)tid;
                for (int q = tid; q < gs * gs; q += kDescThreads, qf += (float)kDescThreads) {
                    const int qy = floor_i((qf + 0.5f) * inv_gs);
                    const int qx = q - qy * gs;
                    const float q11 = g.px_raw(px0 + qx, py0 + qy), q21 = g.px_raw(px0 + qx + 1, py0 + qy);
                    const float q12 = g.px_raw(px0 + qx, py0 + qy + 1), q22 = g.px_raw(px0 + qx + 1, py0 + qy + 1);
                    // the reference's bilinear blend as two lerps (within the
                    // descriptor tolerance)
                    const float r0 = fmaf(fdx, q21 - q11, q11), r1 = fmaf(fdx, q22 - q12, q12);
                    const float b = fmaf(fdy, r1 - r0, r0);
                    grid[qy * gst + (qy & 1) + qx] = b;
                    lo = fminf(lo, b);
                    hi = fmaxf(hi, b);
                }
            }
        } else {
            lo = 0.0f;
            hi = 1.0f;
        }
        // Fixed point: |gx|, |gy| <= range of the sampled values, so every
        // bin is below sqrt(2) * range * total (Gaussian and trilinear
        // weights <= 1 with unit sum); the scale is the largest power of
        // two that keeps that bound under 2^32.
#pragma unroll
        for (int m = 16; m > 0; m >>= 1) {
            lo = fminf(lo, __shfl_xor_sync(0xffffffffu, lo, m));
            hi = fmaxf(hi, __shfl_xor_sync(0xffffffffu, hi, m));
        }
        if ((tid & 31) == 0) {
            red_lo[tid >> 5] = lo;
            red_hi[tid >> 5] = hi;
        }
        __syncthreads();
        lo = fminf(fminf(red_lo[0], red_lo[1]), fminf(red_lo[2], red_lo[3]));
        hi = fmaxf(fmaxf(red_hi[0], red_hi[1]), fmaxf(red_hi[2], red_hi[3]));
        const float range = fmaxf(hi - lo, 1.0f / 65536.0f);
        // and every single contribution (<= sqrt(2) * range) below 2^23,
        // where its rounding to an integer is exact (the subnormal grid of
        // the pair loop, the 2^23 rounding add of the per-sample loop)
        const float per = 1.4143f * range;
        // floor(log2 q) of a positive normal float is its exponent field
        const int fbits = max(0, min(40, min((__float_as_int(4.0e9f / (per * (float)total)) >> 23) - 127,
                                             (__float_as_int(8.0e6f / per) >> 23) - 127)));
        const float to_fix = __int_as_float((127 + fbits) << 23);
        inv_fix = __int_as_float((127 - fbits) << 23);
        // Descriptor samples are interpolated linearly into their bins, so
        // the sample loops are written for speed within the descriptor
        // tolerance: fused multiply-adds, reciprocal products instead of
        // divisions, the hardware's approximate square root and exp2
        // (scale folded in), an arctangent polynomial in units of angle
        // bins (error 1.5e-5 bin) from which the relative angle is binned
        // directly (floor and & 7 give the rem_euclid bins), and the
        // fixed-point rounding fused into the weight product. Each changes a
        // descriptor value by ~1e-5 or less.
        const float inv_bw = 1.0f / bw;
        const float angb = ang * (4.0f / kPi);  // keypoint angle in 45-degree bins
        const float wexp = -1.4426950408889634f / wd;  // exp(-d2/wd) = exp2(d2 * wexp)
        // |rx|, |ry| below lim keep xb, yb inside (-1, 4) after rounding, so
        // every cell index lies in the padded grid (samples within 1e-6
        // of the window edge, whose shares there are ~0, are left out)
        const float lim = __fmul_rn(2.5f, bw) * 0.99999905f;
        unsigned int* hcopy = hist + (tid & 7) * kHistStride;
        const float rad_f = (float)rad;
        // windows that stay inside the level need no per-sample border test
        const bool edge = !(__fadd_rn(xo, -rad_f) >= 0.0f && __fadd_rn(xo, rad_f) < wm1 &&
                            __fadd_rn(yo, -rad_f) >= 0.0f && __fadd_rn(yo, rad_f) < hm1);
        if (use_grid) {
            // Sample pairs: a thread takes the window samples (px, py) and
            // (px + 1, py) and evaluates both with packed f32x2 arithmetic,
            // the same operations per element as one sample alone. A row
            // has rad + 1 pairs: from px = -rad in rows of even grid index
            // (the last pair's second element, px = rad + 1, is outside the
            // window), from px = -rad - 1 in rows of odd grid index (the
            // first pair's first element is outside), so the float pairs
            // of the gradients' grid reads are 8-byte aligned (one 64-bit
            // load each). Pair m = tid + 128 j: the base offset pxb (= px
            // in even rows, px + 1 in odd ones), py (exact small integers
            // in f32), the row parity p and the grid index c of element 0
            // advance by fixed amounts with one row wrap per step.
            const int hp = rad + 1;
            const int q0 = tid / hp, dq = kDescThreads / hp;
            const float dr_f = (float)(2 * (kDescThreads - dq * hp)), dq_f = (float)dq;
            const int dc = dq * gst + 2 * (kDescThreads - dq * hp);
            const int dqp = dq & 1;
            const float wrap_f = (float)(2 * hp);
            // Fixed point on the subnormal grid: a float below 2^-125 is
            // k * 2^-149 and its bit pattern is k, so a contribution scaled
            // by 2^(fbits - 149) and rounded once to the nearest float (the
            // last multiply) has the fixed-point integer as its bits (k <
            // 2^23 by the scale choice): no conversion and no offset to
            // subtract before the atomic. The scale is split so every factor
            // stays a normal float: 2^(fbits - 49) rides in the exponent,
            // exp2(d2 * wexp + fbits - 49) = 2^(fbits - 49) exp(-d2 / wd),
            // and 2^-100 in the two angle weights. (The library is built
            // without flush-to-zero, and mul.rn.f32x2 keeps subnormals.)
            const float fb = (float)(fbits - 49);
            const float2 ca2 = make_float2(ca, ca), sa2 = make_float2(sa, sa), nsa2 = make_float2(-sa, -sa);
            const float2 ib2 = make_float2(inv_bw, inv_bw), half3 = make_float2(1.5f, 1.5f);
            const float2 wexp2 = make_float2(wexp, wexp), fb2 = make_float2(fb, fb);
            const float2 m15 = make_float2(kMagic15, kMagic15), nm15 = make_float2(-kMagic15, -kMagic15);
            const float2 neg1 = make_float2(-1.0f, -1.0f), one2 = make_float2(1.0f, 1.0f);
            constexpr float kAngScale = 7.888609052210118e-31f;  // 2^-100
            const float2 as2 = make_float2(kAngScale, kAngScale), nas2 = make_float2(-kAngScale, -kAngScale);
            const float2 angb2 = make_float2(angb, angb);
            auto pairs = [&](auto edge_tag) {
                constexpr bool kEdge = decltype(edge_tag)::value;
                float pxb = (float)(2 * (tid - q0 * hp)) - rad_f, py = (float)q0 - rad_f;
                int c = (q0 + 1) * gst + 2 * (tid - q0 * hp) + 1;  // odd
                int p = (q0 + 1) & 1;                               // parity of grid row q0 + 1
                for (;; pxb += dr_f, py += dq_f, c += dc, p ^= dqp) {
                    // the wrap to the next row as selects: a branch here
                    // would split the warp for the rest of the step
                    const bool wrap = pxb > rad_f;
                    pxb = wrap ? pxb - wrap_f : pxb;
                    py = wrap ? py + 1.0f : py;
                    c = wrap ? c + 2 : c;
                    p = wrap ? p ^ 1 : p;
                    if (py > rad_f) break;
                    const float px = p ? pxb - 1.0f : pxb;
                    const bool v0 = px >= -rad_f, v1 = px < rad_f;
                    // rows gr - 1 and gr + 1 sit one slot the other way
                    const int cv = c + 1 - 2 * p;
                    const float2 P = make_float2(px, px + 1.0f), Q = make_float2(py, py);
                    const float2 rx = __ffma2_rn(P, ca2, __fmul2_rn(Q, sa2));
                    const float2 ry = __ffma2_rn(P, nsa2, __fmul2_rn(Q, ca2));
                    bool in0 = v0 && fabsf(rx.x) < lim && fabsf(ry.x) < lim;
                    bool in1 = v1 && fabsf(rx.y) < lim && fabsf(ry.y) < lim;
                    if constexpr (kEdge) {
                        const float xs0 = xo + px, ys0 = yo + py, xs1 = xo + P.y;
                        const bool rowin = !(ys0 < 0.0f || ys0 >= hm1);
                        in0 = in0 && rowin && !(xs0 < 0.0f || xs0 >= wm1);
                        in1 = in1 && rowin && !(xs1 < 0.0f || xs1 >= wm1);
                    }
                    // warps whose 64 samples all fall outside skip the rest
                    if (!__any_sync(__activemask(), in0 || in1)) continue;
                    if (!(in0 || in1)) continue;
                    // (left, right) and (above, below) of both elements
                    const float2 gl = *reinterpret_cast<const float2*>(grid + c - 1);
                    const float2 gr = *reinterpret_cast<const float2*>(grid + c + 1);
                    const float2 gu = *reinterpret_cast<const float2*>(grid + cv - gst);
                    const float2 gd = *reinterpret_cast<const float2*>(grid + cv + gst);
                    const float2 gx = __ffma2_rn(gl, neg1, gr);
                    const float2 gy = __ffma2_rn(gu, neg1, gd);
                    const float2 m2 = __ffma2_rn(gx, gx, __fmul2_rn(gy, gy));
                    const float2 ea = __ffma2_rn(__ffma2_rn(P, P, __fmul2_rn(Q, Q)), wexp2, fb2);
                    float2 wm = __fmul2_rn(make_float2(sqrt_approx(m2.x), sqrt_approx(m2.y)),
                                           make_float2(ex2_approx(ea.x), ex2_approx(ea.y)));
                    // an element outside the window adds zero shares to
                    // cell (-1, -1) of its copy
                    wm.x = in0 ? wm.x : 0.0f;
                    wm.y = in1 ? wm.y : 0.0f;
                    const float2 ab = __fadd2_rn(atan2_bins2(gy, gx), make_float2(-angb, -angb));
                    const float2 xb = __ffma2_rn(rx, ib2, half3), yb = __ffma2_rn(ry, ib2, half3);
                    // floors by the 1.5 * 2^23 rounding-down add: the low
                    // bits of tx, ty, ta are the integers
                    const float2 tx = __fadd2_rd(xb, m15), ty = __fadd2_rd(yb, m15), ta = __fadd2_rd(ab, m15);
                    const float2 fx = __ffma2_rn(__fadd2_rn(tx, nm15), neg1, xb);
                    const float2 fy = __ffma2_rn(__fadd2_rn(ty, nm15), neg1, yb);
                    const float2 fa = __ffma2_rn(__fadd2_rn(ta, nm15), neg1, ab);
                    // histogram word of cell (xbi, ybi), bin abi & 7:
                    // ((ybi + 1) * 6 + xbi + 1) * 9 + (abi & 7), from the
                    // float bits (the 0x4B400000 offsets cancel mod 2^32,
                    // 0x4B400000 & 7 == 0)
                    constexpr uint32_t kCellOff = 63u - 63u * 0x4B400000u;
                    uint32_t at0 = __float_as_uint(ty.x) * (uint32_t)(kHistSide * kHistRow) +
                                   __float_as_uint(tx.x) * (uint32_t)kHistRow + kCellOff +
                                   (__float_as_uint(ta.x) & 7u);
                    uint32_t at1 = __float_as_uint(ty.y) * (uint32_t)(kHistSide * kHistRow) +
                                   __float_as_uint(tx.y) * (uint32_t)kHistRow + kCellOff +
                                   (__float_as_uint(ta.y) & 7u);
                    at0 = in0 ? at0 : 0u;
                    at1 = in1 ? at1 : 0u;
                    const float2 wy0 = __fmul2_rn(wm, __ffma2_rn(fy, neg1, one2)), wy1 = __fmul2_rn(wm, fy);
                    const float2 wx0 = __ffma2_rn(fx, neg1, one2);
                    // (1 - fa) * 2^-100 and fa * 2^-100 (exact scalings)
                    const float2 wa0 = __ffma2_rn(fa, nas2, as2), wa1 = __fmul2_rn(fa, as2);
                    unsigned int* h0 = hcopy + at0;
                    unsigned int* h1 = hcopy + at1;
#pragma unroll
                    for (int cc = 0; cc < 4; ++cc) {
                        const float2 wxy = __fmul2_rn((cc & 1) ? fx : wx0, (cc & 2) ? wy1 : wy0);
                        const int off = ((cc & 2) ? kHistSide * kHistRow : 0) + ((cc & 1) ? kHistRow : 0);
                        // the products, rounded to the nearest fixed-point
                        // integer on the subnormal grid, are their own bits
                        const float2 n0 = __fmul2_rn(wxy, wa0), n1 = __fmul2_rn(wxy, wa1);
                        atomicAdd(h0 + off, __float_as_uint(n0.x));
                        atomicAdd(h0 + off + 1, __float_as_uint(n1.x));
                        atomicAdd(h1 + off, __float_as_uint(n0.y));
                        atomicAdd(h1 + off + 1, __float_as_uint(n1.y));
                    }
                }
            };
            if (edge)
                pairs(std::true_type{});
            else
                pairs(std::false_type{});
        } else {
            // Radii above the grid: one sample per thread, four bilinears
            // from the level per sample (the reference's own evaluation).
            for (int k = tid; k < total; k += kDescThreads) {
                const int qy = k / side;
                const float px = (float)(k - qy * side) - rad_f, py = (float)qy - rad_f;
                const float rx = fmaf(ca, px, sa * py);
                const float ry = fmaf(-sa, px, ca * py);
                if (!(fabsf(rx) < lim && fabsf(ry) < lim)) continue;
                const float xs = xo + px, ys = yo + py;
                if (xs < 0.0f || xs >= wm1 || ys < 0.0f || ys >= hm1) continue;
                const float gx =
                    __fsub_rn(g.bilinear(__fadd_rn(xs, 1.0f), ys), g.bilinear(__fsub_rn(xs, 1.0f), ys));
                const float gy =
                    __fsub_rn(g.bilinear(xs, __fadd_rn(ys, 1.0f)), g.bilinear(xs, __fsub_rn(ys, 1.0f)));
                const float mag = sqrt_approx(fmaf(gx, gx, gy * gy));
                const float wm = mag * ex2_approx(fmaf(px, px, py * py) * wexp);
                const float ab = atan2_bins(gy, gx) - angb;  // in [-12, 4]
                const float xb = fmaf(rx, inv_bw, 1.5f), yb = fmaf(ry, inv_bw, 1.5f);
                int xbi, ybi, abi;
                const float xbf = floor_fi(xb, &xbi), ybf = floor_fi(yb, &ybi), abf = floor_fi(ab, &abi);
                const float fx = xb - xbf, fy = yb - ybf, fa = ab - abf;
                const float wa1 = fa * to_fix, wa0 = to_fix - wa1;
                const float wx0 = 1.0f - fx, wx1 = fx;
                const float wy0 = wm * (1.0f - fy), wy1 = wm * fy;
                unsigned int* h0 = hcopy + ((ybi + 1) * kHistSide + (xbi + 1)) * kHistRow + (abi & 7);
#pragma unroll
                for (int cc = 0; cc < 4; ++cc) {
                    const float wxy = ((cc & 1) ? wx1 : wx0) * ((cc & 2) ? wy1 : wy0);
                    unsigned int* hc = h0 + ((cc & 2) ? kHistSide * kHistRow : 0) + ((cc & 1) ? kHistRow : 0);
                    atomicAdd(hc, __float_as_uint(__fmaf_rn(wxy, wa0, kMagic)) - 0x4B000000u);
                    atomicAdd(hc + 1, __float_as_uint(__fmaf_rn(wxy, wa1, kMagic)) - 0x4B000000u);
                }
            }
        }
    }
    __syncthreads();  // the histogram is complete
    // normalize_and_clip_descriptor (src/sift.rs:889-913), one bin per
    // thread; the sums of squares over the four warps in a fixed order
    {
        const int bin = tid;  // (iy * 4 + ix) * 8 + ia
        const int cell = bin >> 3, ia = bin & 7;
        const int at = (((cell >> 2) + 1) * kHistSide + (cell & 3) + 1) * kHistRow + ia;
        unsigned v = 0u;
#pragma unroll
        for (int c = 0; c < kHistCopies; ++c) v += hist[c * kHistStride + at];
        if (ia == 0)
#pragma unroll
            for (int c = 0; c < kHistCopies; ++c) v += hist[c * kHistStride + at + 8];
        float d = __fmul_rn((float)v, inv_fix);
        float ss = __fmul_rn(d, d);
#pragma unroll
        for (int m = 16; m > 0; m >>= 1) ss = __fadd_rn(ss, __shfl_xor_sync(0xffffffffu, ss, m));
        if ((tid & 31) == 0) red_lo[tid >> 5] = ss;
        __syncthreads();
        const float norm = __fsqrt_rn(__fadd_rn(__fadd_rn(red_lo[0], red_lo[1]), __fadd_rn(red_lo[2], red_lo[3])));
        if (!(norm < 1e-8f)) {  // the same for every thread
            d = fminf(__fmul_rn(d, __fdiv_rn(1.0f, norm)), 0.2f);
            float s2 = __fmul_rn(d, d);
#pragma unroll
            for (int m = 16; m > 0; m >>= 1) s2 = __fadd_rn(s2, __shfl_xor_sync(0xffffffffu, s2, m));
            if ((tid & 31) == 0) red_hi[tid >> 5] = s2;
            __syncthreads();
            const float n2 =
                __fsqrt_rn(__fadd_rn(__fadd_rn(red_hi[0], red_hi[1]), __fadd_rn(red_hi[2], red_hi[3])));
            if (!(n2 < 1e-8f)) d = __fmul_rn(d, __fdiv_rn(1.0f, n2));
        }
            dst[bin] = d;
    }
}

// One CTA per oriented keypoint (persistent over the list), describe_one on
// each. Neighbouring samples land in the same bins, so the lanes of a warp
// add into kHistCopies copies of the histogram: adds to one address
// serialise, adds to distinct copies do not. Lane l uses copy l & 7, so the
// lanes sharing a copy hold samples 16 apart (mostly different cells) and
// neighbouring lanes, which often hit the same bin, use copies 4 banks apart;
// picking the copy by l >> 2 instead (4 neighbours per copy) costs 13 % more
// time. The copies are summed in a fixed order; integer sums make the order
// irrelevant.
template <typename TG>
__global__ void __launch_bounds__(kDescThreads, 8) k_descriptor(const TG* __restrict__ arena, EntryTable tab,
                                                              const Keypoint* __restrict__ oriented,
                                                              OctCounters* __restrict__ oc,
                                                              float* __restrict__ desc, uint32_t cap,
                                                              float* __restrict__ hdesc, uint32_t hcap,
                                                              int persist_from) {
    chain_wait();
    __shared__ __align__(16) float grid[kDescGridSide * (kDescGridSide + 1)];
    __shared__ __align__(16) unsigned int hist[kHistCopies * kHistStride];
    __shared__ float red_lo[kDescThreads / 32], red_hi[kDescThreads / 32];
    const int tid = threadIdx.x;
    const uint32_t base = oc->out_base;
    uint32_t n = oc->n_ori;
    if (base >= cap) n = 0;
    else if (n > cap - base) n = cap - base;
    // Keypoints differ ~4x in window area: they come from a queue. Thread 0
    // claims the next item while the CTA works on the current one (slot
    // next[p ^ 1]), unless the CTA retires after the current one.
    __shared__ uint32_t next[2];
    const bool persist = (int)blockIdx.x >= persist_from;
    if (tid == 0) next[0] = atomicAdd(&oc->next_desc, 1u);
    for (int taken = 0, p = 0;; ++taken, p ^= 1) {
        __syncthreads();  // next[p] is visible, the grid and histogram are free
        const uint32_t cur = next[p];
        if (cur >= n) break;
        const bool more = persist || taken + 1 < kDescBudget;
        uint32_t claim = n;
        if (tid == 0 && more) claim = atomicAdd(&oc->next_desc, 1u);
        // the queue runs from the last keypoint: an octave's list is in layer
        // order, so the largest windows go first and the smallest make the
        // tail of the stage
        const uint32_t i = base + (n - 1 - cur);
        const Keypoint kp = oriented[i];
        // keypoints below hcap straight into the host call's mapped buffer
        describe_one<TG>(arena, tab, kp, grid, hist, red_lo, red_hi, (i < hcap ? hdesc : desc) + (size_t)i * kDescLen);
        if (tid == 0) next[p ^ 1] = claim;
    }
}


}  // namespace

template <typename TG>
int launch_orientation(const TG* arena, const EntryTable& tab, const float* lut255, const Keypoint* refined_at,
                       const uint32_t* keep, uint32_t ncap, OctCounters* oc, float* ori_angle, uint32_t* ori_count,
                       int grid, int persist_ctas, cudaStream_t st) {
    if (launch_chained(k_orientation<TG>, grid, dim3(32, kOriWarps), 0, st, arena, tab, lut255, refined_at, keep, ncap,
                       oc, ori_angle, ori_count, std::max(grid - persist_ctas, 0)) != cudaSuccess)
        return -1;
    return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
}

int launch_orient_emit(const Keypoint* refined_at, uint32_t ncap, int o, Counters* ctr, const float* ori_angle,
                       const uint32_t* ori_count, const uint32_t* ori_off, Keypoint* oriented, uint32_t cap,
                       cudaStream_t st) {
    if (launch_chained(k_orient_emit, 152, 256, 0, st, refined_at, ncap, o, ctr, ori_angle, ori_count, ori_off,
                       oriented, cap) != cudaSuccess)
        return -1;
    return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
}

template <typename TG>
int launch_descriptor(const TG* arena, const EntryTable& tab, const Keypoint* oriented,
                      OctCounters* oc, float* desc, uint32_t cap, float* hdesc, uint32_t hcap, int grid,
                      int persist_ctas, cudaStream_t st) {
    if (!hdesc) hcap = 0;
    if (launch_chained(k_descriptor<TG>, grid, kDescThreads, 0, st, arena, tab, oriented, oc, desc, cap, hdesc,
                       hcap, std::max(grid - persist_ctas, 0)) != cudaSuccess)
        return -1;
    return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
}

#define SIFT_INST(TG)                                                                                              \
    template int launch_orientation<TG>(const TG*, const EntryTable&, const float*, const Keypoint*,               \
                                        const uint32_t*,                                                           \
                                        uint32_t, OctCounters*, float*, uint32_t*, int, int, cudaStream_t);        \
    template int launch_descriptor<TG>(const TG*, const EntryTable&, const Keypoint*, OctCounters*,                \
                                       float*, uint32_t, float*, uint32_t, int, int, cudaStream_t);
SIFT_INST(float)
SIFT_INST(__half)
SIFT_INST(uint8_t)
#undef SIFT_INST

}  // namespace sift
