// match.cu — brute-force descriptor matching: for every query descriptor the
// nearest and second-nearest train descriptor by Euclidean distance, the
// input of Lowe's ratio test. Not part of the reference crate; it consumes
// the 128-float descriptors that detect_and_compute returns.
//
// Squared distances are |q|^2 + |t|^2 - 2 q.t. A 128-query tile stays in
// shared memory while 64-descriptor train tiles stream through it; TF32
// tensor-core products pick each query's 4 best candidates per train chunk,
// which are re-ranked with exact f32 dot products. Work items are (query
// tile, train chunk) pairs taken from an atomic queue by a grid of one wave of
// CTAs; a second kernel folds the chunks. Ties go to the lower train index, so
// the result does not depend on the chunking or the order items are taken in.
#include <algorithm>

#include "sift_internal.cuh"

namespace sift {
namespace {

constexpr int kMT = 64;  // train descriptors per tile (the chunk unit)
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

// The dot products of a 128-query x 64-train tile come from
// TF32 mma.sync (m16n8k8, f32 accumulate; 8 warps of 32 x 32): approximate
// squared distances that only select each query's 4 best candidates of the
// chunk (a running list per row behind a threshold test). The candidates are
// then re-ranked with exact f32 distances computed as in the f32 kernel (the
// dot product as an FMA chain in index order), so the returned best two are
// the f32 result unless the TF32 error (relative ~1e-3 on a dot product)
// pushes a true best-two outside the 4 candidates.
constexpr int kTQ = 128, kTT = 64;  // CTA tile: queries x train
constexpr int kTS = kD + 4;         // shared row stride (floats): fragment loads in 32 banks
constexpr int kTThreads = 256;      // warps 4 (queries) x 2 (train), 32 x 32 each
constexpr int kTCtasPerSm = 2;      // 101 KB of shared memory per CTA
constexpr int kCand = 4;

struct Cand4 {
    float d[kCand];
    int i[kCand];
};

__device__ __forceinline__ void cand_init(Cand4& c) {
#pragma unroll
    for (int k = 0; k < kCand; ++k) {
        c.d[k] = INFINITY;
        c.i[k] = -1;
    }
}

// sorted insertion (ties to the lower index); the caller tests d < c.d[3]
__device__ __forceinline__ void cand_push(Cand4& c, float d, int i) {
#pragma unroll
    for (int k = kCand - 1; k >= 0; --k) {
        const bool above = k > 0 && before(d, i, c.d[k - 1], c.i[k - 1]);
        if (before(d, i, c.d[k], c.i[k])) {
            c.d[k] = above ? c.d[k - 1] : d;
            c.i[k] = above ? c.i[k - 1] : i;
        }
    }
}

__device__ __forceinline__ void mma_tf32(float (&c)[4], const uint32_t (&a)[4], const uint32_t (&b)[2]) {
    asm volatile(
        "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// rows [row0, row0 + rows) of x into tile[r][k] (row stride kTS); past n: zeros
__device__ __forceinline__ void stage_rows(const float* __restrict__ x, uint32_t n, uint32_t row0, int rows,
                                           float* tile) {
    for (int q = threadIdx.x; q < rows * (kD / 4); q += kTThreads) {
        const int r = q / (kD / 4), k4 = q % (kD / 4);
        float4 v = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        if (row0 + r < n) v = reinterpret_cast<const float4*>(x + (size_t)(row0 + r) * kD)[k4];
        *reinterpret_cast<float4*>(tile + r * kTS + 4 * k4) = v;
    }
}

__global__ void __launch_bounds__(kTThreads) k_match_tc(const float* __restrict__ q, const float* __restrict__ qn,
                                                        uint32_t nq, const float* __restrict__ t,
                                                        const float* __restrict__ tn, uint32_t nt,
                                                        uint32_t chunk_tiles, uint32_t n_chunks,
                                                        uint32_t* __restrict__ next, float4* __restrict__ part) {
    extern __shared__ __align__(16) float sm[];
    float* qs = sm;                                              // [kTQ][kTS]
    float* ts = sm + kTQ * kTS;                                  // [kTT][kTS]
    float* xd = ts + kTT * kTS;                                  // [2][kTQ][kCand] candidate exchange
    int* xi = reinterpret_cast<int*>(xd + 2 * kTQ * kCand);      // [2][kTQ][kCand]
    __shared__ uint32_t item_s;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int g = lane >> 2, tq = lane & 3;  // mma fragment row group, thread in group
    const int wq = warp & 3, wt = warp >> 2;
    const uint32_t n_tiles = (nt + kTT - 1) / kTT;
    const uint32_t items = ((nq + kTQ - 1) / kTQ) * n_chunks;
    uint32_t staged = 0xffffffffu;
    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0) item_s = atomicAdd(next, 1u);
        __syncthreads();
        const uint32_t item = item_s;
        if (item >= items) break;
        const uint32_t qt = item / n_chunks, chunk = item - qt * n_chunks;
        const uint32_t q0 = qt * kTQ;
        if (qt != staged) {
            stage_rows(q, nq, q0, kTQ, qs);
            staged = qt;
        }
        // this thread's 4 rows: mi in {0, 1} x {g, g + 8}
        float qnr[4];
        Cand4 cand[4];
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            const uint32_t row = q0 + wq * 32 + (r >> 1) * 16 + g + (r & 1) * 8;
            qnr[r] = row < nq ? qn[row] : 0.0f;
            cand_init(cand[r]);
        }
        const uint32_t tile_lo = chunk * chunk_tiles, tile_hi = min(tile_lo + chunk_tiles, n_tiles);
        for (uint32_t tt = tile_lo; tt < tile_hi; ++tt) {
            const uint32_t t0 = tt * kTT;
            __syncthreads();
            stage_rows(t, nt, t0, kTT, ts);
            __syncthreads();
            float acc[2][4][4];
#pragma unroll
            for (int mi = 0; mi < 2; ++mi)
#pragma unroll
                for (int ni = 0; ni < 4; ++ni)
#pragma unroll
                    for (int e = 0; e < 4; ++e) acc[mi][ni][e] = 0.0f;
            const float* qa = qs + (wq * 32 + g) * kTS + tq;
            const float* tb = ts + (wt * 32 + g) * kTS + tq;
#pragma unroll 4
            for (int kk = 0; kk < kD; kk += 8) {
                uint32_t a[2][4], b[4][2];
#pragma unroll
                for (int mi = 0; mi < 2; ++mi) {
                    const float* p = qa + mi * 16 * kTS + kk;
                    a[mi][0] = __float_as_uint(p[0]);
                    a[mi][1] = __float_as_uint(p[8 * kTS]);
                    a[mi][2] = __float_as_uint(p[4]);
                    a[mi][3] = __float_as_uint(p[8 * kTS + 4]);
                }
#pragma unroll
                for (int ni = 0; ni < 4; ++ni) {
                    const float* p = tb + ni * 8 * kTS + kk;
                    b[ni][0] = __float_as_uint(p[0]);
                    b[ni][1] = __float_as_uint(p[4]);
                }
#pragma unroll
                for (int mi = 0; mi < 2; ++mi)
#pragma unroll
                    for (int ni = 0; ni < 4; ++ni) mma_tf32(acc[mi][ni], a[mi], b[ni]);
            }
            // accumulator (mi, ni, e): row wq*32 + mi*16 + g + 8*(e >> 1), column wt*32 + ni*8 + 2*tq + (e & 1)
#pragma unroll
            for (int ni = 0; ni < 4; ++ni)
#pragma unroll
                for (int c = 0; c < 2; ++c) {
                    const uint32_t col = t0 + wt * 32 + ni * 8 + 2 * tq + c;
                    if (col >= nt) continue;
                    const float tnc = tn[col];
#pragma unroll
                    for (int r = 0; r < 4; ++r) {
                        const float d = fmaf(-2.0f, acc[r >> 1][ni][2 * (r & 1) + c], qnr[r] + tnc);
                        if (d < cand[r].d[kCand - 1] || (d == cand[r].d[kCand - 1] && (int)col < cand[r].i[kCand - 1]))
                            cand_push(cand[r], d, (int)col);
                    }
                }
        }
        // merge the 4 lanes of a row group (tq), then the two column warps
#pragma unroll
        for (int r = 0; r < 4; ++r) {
#pragma unroll
            for (int m = 1; m <= 2; m <<= 1) {
                Cand4 o;
#pragma unroll
                for (int k = 0; k < kCand; ++k) {
                    o.d[k] = __shfl_xor_sync(0xffffffffu, cand[r].d[k], m);
                    o.i[k] = __shfl_xor_sync(0xffffffffu, cand[r].i[k], m);
                }
#pragma unroll
                for (int k = 0; k < kCand; ++k)
                    if (before(o.d[k], o.i[k], cand[r].d[kCand - 1], cand[r].i[kCand - 1])) cand_push(cand[r], o.d[k], o.i[k]);
            }
            const int row = wq * 32 + (r >> 1) * 16 + g + (r & 1) * 8;
            if (tq == 0)
#pragma unroll
                for (int k = 0; k < kCand; ++k) {
                    xd[(wt * kTQ + row) * kCand + k] = cand[r].d[k];
                    xi[(wt * kTQ + row) * kCand + k] = cand[r].i[k];
                }
        }
        __syncthreads();
        // exact re-ranking: thread pair (2 row, 2 row + 1) per query row, two
        // candidates each out of the union of both column warps' lists
        {
            const int row = threadIdx.x >> 1, half = threadIdx.x & 1;
            Cand4 u;
            cand_init(u);
#pragma unroll
            for (int w = 0; w < 2; ++w)
#pragma unroll
                for (int k = 0; k < kCand; ++k) {
                    const float d = xd[(w * kTQ + row) * kCand + k];
                    const int i = xi[(w * kTQ + row) * kCand + k];
                    if (i >= 0 && before(d, i, u.d[kCand - 1], u.i[kCand - 1])) cand_push(u, d, i);
                }
            const uint32_t qi = q0 + row;
            Best2 b{INFINITY, INFINITY, -1, -1};
            if (qi < nq) {
                const float qnq = qn[qi];
                const float4* qv = reinterpret_cast<const float4*>(qs + row * kTS);
#pragma unroll
                for (int k = 0; k < 2; ++k) {
                    const int ci = u.i[2 * half + k];
                    if (ci < 0) continue;
                    const float4* tv = reinterpret_cast<const float4*>(t + (size_t)ci * kD);
                    float dot = 0.0f;
#pragma unroll 8
                    for (int k4 = 0; k4 < kD / 4; ++k4) {
                        const float4 a = qv[k4], c = tv[k4];
                        dot = fmaf(a.x, c.x, dot);
                        dot = fmaf(a.y, c.y, dot);
                        dot = fmaf(a.z, c.z, dot);
                        dot = fmaf(a.w, c.w, dot);
                    }
                    push(b, fmaf(-2.0f, dot, qnq + tn[ci]), ci);
                }
            }
            Best2 o;
            o.d1 = __shfl_xor_sync(0xffffffffu, b.d1, 1);
            o.d2 = __shfl_xor_sync(0xffffffffu, b.d2, 1);
            o.i1 = __shfl_xor_sync(0xffffffffu, b.i1, 1);
            o.i2 = __shfl_xor_sync(0xffffffffu, b.i2, 1);
            b = fold(b, o);
            if (half == 0 && qi < nq)
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
    const size_t smem = sizeof(float) * ((kTQ + kTT) * kTS + 2 * kTQ * kCand) + sizeof(int) * 2 * kTQ * kCand;
    if (cudaFuncSetAttribute(k_match_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return -1;
    const uint32_t items = ((nq + kTQ - 1) / kTQ) * n_chunks;
    const uint32_t grid = std::min<uint32_t>(items, 152u * kTCtasPerSm);
    k_match_tc<<<grid, kTThreads, smem, st>>>(d_q, qn, nq, d_t, tn, nt, chunk_tiles, n_chunks, next, part);
    k_match_fold<<<(nq + 255) / 256, 256, 0, st>>>(part, nq, n_chunks, d_out);
    return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace sift
