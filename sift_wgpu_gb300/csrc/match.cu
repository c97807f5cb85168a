// match.cu — brute-force descriptor matching: for every query descriptor the
// nearest and second-nearest train descriptor by Euclidean distance, the
// input of Lowe's ratio test. Not part of the reference crate; it consumes
// the 128-float descriptors that detect_and_compute returns.
//
// Squared distances are |q|^2 + |t|^2 - 2 q.t in f32, the dot products from a
// register-tiled product of a 64-query tile (resident in shared memory) and
// 64-descriptor train tiles streamed through shared memory: each thread owns
// 4 queries x 4 train descriptors (16 accumulators, two 16-byte shared loads
// per 16 fused multiply-adds) and keeps a running best-two per query. Work
// items are (query tile, train chunk) pairs taken from an atomic queue by a
// grid of one wave of CTAs (no partial last wave); a second kernel folds the
// chunks. Ties go to the lower train index, so the result does not depend on
// the chunking or the order items are taken in.
#include <algorithm>

#include "sift_internal.cuh"

namespace sift {
namespace {

constexpr int kMQ = 64;               // queries per CTA
constexpr int kMT = 64;               // train descriptors per tile
constexpr int kMS = kMQ + 4;          // shared row stride (floats): 16-byte aligned rows
constexpr int kMThreads = 256;        // 16 x 16 threads, 4 x 4 outputs each
constexpr int kMCtasPerSm = 3;        // 70 KB of shared memory per CTA
constexpr int kD = kDescLen;

struct Best2 {
    float d1, d2;
    int i1, i2;
};

__device__ __forceinline__ bool before(float d, int i, float e, int j) { return d < e || (d == e && i < j); }

__device__ __forceinline__ void push(Best2& b, float d, int i) {
    if (before(d, i, b.d1, b.i1)) {
        b.d2 = b.d1;
        b.i2 = b.i1;
        b.d1 = d;
        b.i1 = i;
    } else if (before(d, i, b.d2, b.i2)) {
        b.d2 = d;
        b.i2 = i;
    }
}

// The best two of two best-two lists.
__device__ __forceinline__ Best2 fold(const Best2& a, const Best2& b) {
    Best2 r;
    if (before(a.d1, a.i1, b.d1, b.i1)) {
        r.d1 = a.d1;
        r.i1 = a.i1;
        const bool sa = before(a.d2, a.i2, b.d1, b.i1);
        r.d2 = sa ? a.d2 : b.d1;
        r.i2 = sa ? a.i2 : b.i1;
    } else {
        r.d1 = b.d1;
        r.i1 = b.i1;
        const bool sb = before(b.d2, b.i2, a.d1, a.i1);
        r.d2 = sb ? b.d2 : a.d1;
        r.i2 = sb ? b.i2 : a.i1;
    }
    return r;
}

// Squared norm of each descriptor row, summed in index order.
__global__ void k_sq_norms(const float* __restrict__ x, uint32_t n, float* __restrict__ out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4* r = reinterpret_cast<const float4*>(x + (size_t)i * kD);
    float s = 0.0f;
#pragma unroll 8
    for (int k = 0; k < kD / 4; ++k) {
        const float4 v = r[k];
        s = fmaf(v.x, v.x, s);
        s = fmaf(v.y, v.y, s);
        s = fmaf(v.z, v.z, s);
        s = fmaf(v.w, v.w, s);
    }
    out[i] = s;
}

// Rows [row0, row0 + 64) of x (n rows) into tile[k][r] (k-major, stride kMS);
// rows past n become zeros. Lanes take consecutive rows, so the transposing
// stores hit distinct banks.
__device__ __forceinline__ void stage_tile(const float* __restrict__ x, uint32_t n, uint32_t row0, float* tile) {
    for (int q = threadIdx.x; q < kMQ * (kD / 4); q += kMThreads) {
        const int r = q % kMQ, k4 = q / kMQ;
        float4 v = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        if (row0 + r < n) v = reinterpret_cast<const float4*>(x + (size_t)(row0 + r) * kD)[k4];
        tile[(4 * k4 + 0) * kMS + r] = v.x;
        tile[(4 * k4 + 1) * kMS + r] = v.y;
        tile[(4 * k4 + 2) * kMS + r] = v.z;
        tile[(4 * k4 + 3) * kMS + r] = v.w;
    }
}

// Items (query tile, train chunk) from the queue *next; for each, the best
// two per query of the tile over the chunk's train tiles:
// part[chunk * nq + q] = {d1, i1, d2, i2} (squared distances, index bits).
__global__ void __launch_bounds__(kMThreads) k_match_tiles(const float* __restrict__ q, const float* __restrict__ qn,
                                                           uint32_t nq, const float* __restrict__ t,
                                                           const float* __restrict__ tn, uint32_t nt,
                                                           uint32_t chunk_tiles, uint32_t n_chunks,
                                                           uint32_t* __restrict__ next, float4* __restrict__ part) {
    extern __shared__ __align__(16) float sm[];
    float* qs = sm;             // [kD][kMS]
    float* ts = sm + kD * kMS;  // [kD][kMS]
    __shared__ uint32_t item_s;
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    const uint32_t n_tiles = (nt + kMT - 1) / kMT;
    const uint32_t items = ((nq + kMQ - 1) / kMQ) * n_chunks;
    uint32_t staged = 0xffffffffu;  // query tile in qs
    for (;;) {
        __syncthreads();  // the previous item's reads of qs, ts and item_s are done
        if (threadIdx.x == 0) item_s = atomicAdd(next, 1u);
        __syncthreads();
        const uint32_t item = item_s;
        if (item >= items) break;
        const uint32_t qt = item / n_chunks, chunk = item - qt * n_chunks;
        const uint32_t q0 = qt * kMQ;
        if (qt != staged) {
            stage_tile(q, nq, q0, qs);
            staged = qt;
        }
        float qnr[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) qnr[i] = q0 + 4 * ty + i < nq ? qn[q0 + 4 * ty + i] : 0.0f;
        Best2 best[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) best[i] = Best2{INFINITY, INFINITY, -1, -1};
        const uint32_t tile_lo = chunk * chunk_tiles, tile_hi = min(tile_lo + chunk_tiles, n_tiles);
        for (uint32_t tt = tile_lo; tt < tile_hi; ++tt) {
            const uint32_t t0 = tt * kMT;
            __syncthreads();  // the previous tile's reads of ts are done (and qs is staged)
            stage_tile(t, nt, t0, ts);
            __syncthreads();
            float acc[4][4];
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[i][j] = 0.0f;
#pragma unroll 8
            for (int k = 0; k < kD; ++k) {
                const float4 a = *reinterpret_cast<const float4*>(qs + k * kMS + 4 * ty);
                const float4 b = *reinterpret_cast<const float4*>(ts + k * kMS + 4 * tx);
                const float av[4] = {a.x, a.y, a.z, a.w}, bv[4] = {b.x, b.y, b.z, b.w};
#pragma unroll
                for (int i = 0; i < 4; ++i)
#pragma unroll
                    for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(av[i], bv[j], acc[i][j]);
            }
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const uint32_t ti = t0 + 4 * tx + j;
                if (ti >= nt) break;
                const float tnj = tn[ti];
#pragma unroll
                for (int i = 0; i < 4; ++i) push(best[i], fmaf(-2.0f, acc[i][j], qnr[i] + tnj), (int)ti);
            }
        }
        // fold the 16 column threads of each query row (lanes of one half-warp)
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            Best2 b = best[i];
#pragma unroll
            for (int m = 8; m > 0; m >>= 1) {
                Best2 o;
                o.d1 = __shfl_xor_sync(0xffffffffu, b.d1, m);
                o.d2 = __shfl_xor_sync(0xffffffffu, b.d2, m);
                o.i1 = __shfl_xor_sync(0xffffffffu, b.i1, m);
                o.i2 = __shfl_xor_sync(0xffffffffu, b.i2, m);
                b = fold(b, o);
            }
            const uint32_t qi = q0 + 4 * ty + i;
            if (tx == 0 && qi < nq)
                part[(size_t)chunk * nq + qi] = make_float4(b.d1, __int_as_float(b.i1), b.d2, __int_as_float(b.i2));
        }
    }
}

// Fold the chunks of each query in chunk order and convert to distances.
__global__ void k_match_fold(const float4* __restrict__ part, uint32_t nq, uint32_t splits,
                             SiftCudaMatch* __restrict__ out) {
    const uint32_t qi = blockIdx.x * blockDim.x + threadIdx.x;
    if (qi >= nq) return;
    Best2 b{INFINITY, INFINITY, -1, -1};
    for (uint32_t s = 0; s < splits; ++s) {
        const float4 p = part[(size_t)s * nq + qi];
        b = fold(b, Best2{p.x, p.z, __float_as_int(p.y), __float_as_int(p.w)});
    }
    SiftCudaMatch m;
    m.train_idx = b.i1;
    m.distance = b.i1 >= 0 ? sqrtf(fmaxf(b.d1, 0.0f)) : INFINITY;
    m.second_idx = b.i2;
    m.second_distance = b.i2 >= 0 ? sqrtf(fmaxf(b.d2, 0.0f)) : INFINITY;
    out[qi] = m;
}

// Train chunks of at least 16 tiles (1024 descriptors), at most 64 chunks.
void match_chunks(uint32_t nt, uint32_t* chunk_tiles, uint32_t* n_chunks) {
    const uint32_t tt = std::max<uint32_t>((nt + kMT - 1) / kMT, 1u);
    *chunk_tiles = std::max<uint32_t>(16u, (tt + 63) / 64);
    *n_chunks = (tt + *chunk_tiles - 1) / *chunk_tiles;
}

size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

}  // namespace

size_t match_scratch_bytes(uint32_t nq, uint32_t nt) {
    uint32_t ct, nc;
    match_chunks(nt, &ct, &nc);
    return align256((size_t)nq * 4) + align256((size_t)nt * 4) + 256 + (size_t)nc * nq * sizeof(float4);
}

int launch_match(const float* d_q, uint32_t nq, const float* d_t, uint32_t nt, SiftCudaMatch* d_out, void* scratch,
                 cudaStream_t st) {
    if (nq == 0) return 0;
    uint32_t chunk_tiles, n_chunks;
    match_chunks(nt, &chunk_tiles, &n_chunks);
    char* p = static_cast<char*>(scratch);
    float* qn = reinterpret_cast<float*>(p);
    p += align256((size_t)nq * 4);
    float* tn = reinterpret_cast<float*>(p);
    p += align256((size_t)nt * 4);
    uint32_t* next = reinterpret_cast<uint32_t*>(p);
    float4* part = reinterpret_cast<float4*>(p + 256);
    k_sq_norms<<<(nq + 255) / 256, 256, 0, st>>>(d_q, nq, qn);
    if (nt) k_sq_norms<<<(nt + 255) / 256, 256, 0, st>>>(d_t, nt, tn);
    if (cudaMemsetAsync(next, 0, sizeof(uint32_t), st) != cudaSuccess) return -1;
    const size_t smem = sizeof(float) * 2 * kD * kMS;
    if (cudaFuncSetAttribute(k_match_tiles, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return -1;
    const uint32_t items = ((nq + kMQ - 1) / kMQ) * n_chunks;
    const uint32_t grid = std::min<uint32_t>(items, 152u * kMCtasPerSm);
    k_match_tiles<<<grid, kMThreads, smem, st>>>(d_q, qn, nq, d_t, tn, nt, chunk_tiles, n_chunks, next, part);
    k_match_fold<<<(nq + 255) / 256, 256, 0, st>>>(part, nq, n_chunks, d_out);
    return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace sift
