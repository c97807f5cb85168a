// match.cu — brute-force descriptor matching: for every query descriptor the
// nearest and second-nearest train descriptor by Euclidean distance, the
// input of Lowe's ratio test. Not part of the reference crate; it consumes
// the 128-float descriptors that detect_and_compute returns.
//
// Squared distances are |q|^2 + |t|^2 - 2 q.t. The products q.t run on the
// 5th-generation tensor cores (tcgen05, TF32 operands, f32 accumulators in
// tensor memory) over TMA-staged 128-descriptor tiles; they only select each
// query's 4 best candidates per train chunk, which are re-ranked with exact
// f32 dot products. (query tile, train chunk) items are CTAs; a second kernel
// folds the chunks. Ties go to the lower train index, so the result does not
// depend on the chunking.
#include <cuda.h>

#include <algorithm>

#include "sift_internal.cuh"
#include "tma.cuh"

namespace sift {
namespace {

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
__global__ void k_sq_norms(const float* __restrict__ x, uint32_t n, float* __restrict__ out, uint32_t n_out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_out) return;
    if (i >= n) {  // padding: never a candidate
        out[i] = INFINITY;
        return;
    }
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

constexpr int kCand = 4;

// ---------------------------------------------------------------------------
// 5th-generation tensor cores (tcgen05) with TMA-staged operands.
//
// One CTA per (query tile, train chunk) item. The query tile (128 rows x 128
// floats, 64 KB) and the train tiles (128 rows, double-buffered) are loaded
// by TMA (cp.async.bulk.tensor, 128-byte swizzle: four 32-float boxes per
// tile) into the K-major layout the MMA reads. One thread issues
// tcgen05.mma.kind::tf32 (M = 128 queries, N = 128 train, K = 8 per
// instruction, 16 per tile) into one of two 128-column f32 accumulators in
// tensor memory, so the epilogue of one tile overlaps the products of the
// next. The epilogue warps own the accumulator's lanes: a thread reads one
// query row's products of half the tile with tcgen05.ld, ranks the columns by
// |t|^2 - 2 q.t and keeps the row's 4 best candidates of the chunk; the two
// halves' lists are merged and re-ranked with exact f32 dot products.
//
// Roles: warps 0-7 epilogue (warp w: tensor-memory lanes 32 (w % 4) .., half
// w / 4 of each tile's columns), warp 8 TMA producer, warp 9 MMA issuer and
// tensor-memory owner. Every mbarrier
// wait is bounded; a wait that runs out sets the error word and the CTA
// leaves through the same exit (tensor memory is always freed).
constexpr int kUM = 128, kUN = 128;                   // MMA M (queries) and N (train rows per tile)
constexpr int kUThreads = 320;  // warps 0-7 epilogue, 8 TMA, 9 MMA
constexpr uint32_t kUAtom = kUM * 128;                // one 32-float K slice of a 128-row tile: 16 KB
constexpr uint32_t kUTile = 4 * kUAtom;               // 64 KB
constexpr uint32_t kUSmem = 3 * kUTile + 8192 + 1024;  // query tile, two train stages, barriers and
                                                       // epilogue buffers, alignment
constexpr uint32_t kUTmemCols = 2 * kUN;
constexpr uint32_t kUSpin = 1u << 26;                 // bounded waits (~seconds)

// bounded mbarrier waits of this kernel
__device__ __forceinline__ bool mbar_wait(uint64_t* b, uint32_t parity) { return sift::mbar_wait(b, parity, kUSpin); }
// Shared-memory matrix descriptor of a K-major operand with 128-byte
// swizzling: 8-row groups of 128-byte rows, 1024 bytes apart.
__device__ __forceinline__ uint64_t umma_desc(uint32_t saddr) {
    return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)1 << 16) | ((uint64_t)(1024 >> 4) << 32) |
           ((uint64_t)1 << 46) | ((uint64_t)2 << 61);
}
// Instruction descriptor: D f32, A and B tf32, both K-major, N = 128, M = 128.
constexpr uint32_t kUIdesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(kUN >> 3) << 17) | ((uint32_t)(kUM >> 4) << 24);

__device__ __forceinline__ void umma_tf32(uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.u32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}" ::"r"(
            dtmem),
        "l"(adesc), "l"(bdesc), "r"(kUIdesc), "r"(accumulate)
        : "memory");
}
__device__ __forceinline__ void umma_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,"
        "%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void epi_barrier() { asm volatile("bar.sync 1, 256;" ::: "memory"); }

__global__ void __launch_bounds__(kUThreads, 1)
    k_match_umma(const __grid_constant__ CUtensorMap tmq, const __grid_constant__ CUtensorMap tmt,
                 const float* __restrict__ q, const float* __restrict__ qn, uint32_t nq, const float* __restrict__ t,
                 const float* __restrict__ tn, uint32_t nt, uint32_t chunk_tiles, uint32_t n_chunks,
                 float4* __restrict__ part, uint32_t* __restrict__ err) {
    extern __shared__ uint8_t usm_raw[];
    uint8_t* usm = reinterpret_cast<uint8_t*>(((uintptr_t)usm_raw + 1023) & ~(uintptr_t)1023);
    uint8_t* qs = usm;                     // [4 K slices][128 rows][128 B], swizzled
    uint8_t* ts = usm + kUTile;            // [2 stages] of the same
    uint64_t* bars = reinterpret_cast<uint64_t*>(usm + 3 * kUTile);
    uint64_t* q_full = bars;               // query tile landed
    uint64_t* t_full = bars + 1;           // [2] train stage landed
    uint64_t* t_empty = bars + 3;          // [2] train stage consumed by the MMAs
    uint64_t* acc_full = bars + 5;         // [2] accumulator complete
    uint64_t* acc_empty = bars + 7;        // [2] accumulator read by the epilogue
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 9);
    uint32_t* bad = tmem_slot + 1;         // a wait of this CTA ran out
    float* tnb = reinterpret_cast<float*>(usm + 3 * kUTile + 1024);  // [2][kUN] train norms of a tile
    float* mrg_d = tnb + 2 * kUN;                                     // [kUM][4] candidates of the second half
    int* mrg_i = reinterpret_cast<int*>(mrg_d + kUM * 4);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const uint32_t n_tiles_all = (nt + kUN - 1) / kUN;
    const uint32_t qt = blockIdx.x / n_chunks, chunk = blockIdx.x - qt * n_chunks;
    const uint32_t q0 = qt * kUM;
    const uint32_t tile_lo = chunk * chunk_tiles;
    const uint32_t tile_hi = min(tile_lo + chunk_tiles, n_tiles_all);
    const int ntile = tile_hi > tile_lo ? (int)(tile_hi - tile_lo) : 0;
    if (tid == 0) {
        mbar_init(q_full, 1);
        for (int i = 0; i < 2; ++i) {
            mbar_init(t_full + i, 1);
            mbar_init(t_empty + i, 1);
            mbar_init(acc_full + i, 1);
            mbar_init(acc_empty + i, 256);
        }
        *bad = 0u;
        mbar_init_fence();
    }
    if (warp == 9) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(kUTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;

    if (warp == 8) {
        if (lane == 0) {
            // query tile, then the chunk's train tiles through two stages
            mbar_expect_tx(q_full, kUTile);
            for (int a = 0; a < 4; ++a) tma_load_2d(qs + a * kUAtom, &tmq, 32 * a, (int)q0, q_full);
            int issued = 0;
            for (int j = 0; j < ntile; ++j) {
                const int st = j & 1;
                if (j >= 2 && !mbar_wait(t_empty + st, ((j >> 1) - 1) & 1)) {
                    atomicOr(bad, 1u);
                    break;
                }
                const int t0 = (int)(tile_lo + j) * kUN;
                mbar_expect_tx(t_full + st, kUTile);
                for (int a = 0; a < 4; ++a) tma_load_2d(ts + st * kUTile + a * kUAtom, &tmt, 32 * a, t0, t_full + st);
                issued = j + 1;
            }
            // no copy of this CTA may still be landing when it exits (on the
            // normal path these phases completed long ago)
            bool landed = mbar_wait(q_full, 0);
            for (int j = issued - 2 < 0 ? 0 : issued - 2; j < issued; ++j)
                landed = mbar_wait(t_full + (j & 1), (j >> 1) & 1) && landed;
            if (!landed) atomicOr(bad, 1u);
        }
    } else if (warp == 9) {
        if (lane == 0) {
            bool ok = mbar_wait(q_full, 0);
            for (int j = 0; ok && j < ntile; ++j) {
                const int st = j & 1, b = j & 1;
                ok = mbar_wait(t_full + st, (j >> 1) & 1);
                if (ok && j >= 2) ok = mbar_wait(acc_empty + b, ((j >> 1) - 1) & 1);
                if (!ok) break;
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const uint32_t qa = smem_u32(qs), ta = smem_u32(ts + st * kUTile);
#pragma unroll
                for (int k = 0; k < kD / 8; ++k) {
                    // K slice k / 4, 32-byte step k % 4 inside the swizzled 128-byte rows
                    const uint32_t off = (uint32_t)(k >> 2) * kUAtom + (uint32_t)(k & 3) * 32u;
                    umma_tf32(tmem + (uint32_t)(b * kUN), umma_desc(qa + off), umma_desc(ta + off), k > 0 ? 1u : 0u);
                }
                umma_commit(t_empty + st);
                umma_commit(acc_full + b);
            }
            if (!ok) atomicOr(bad, 1u);
        }
    } else {
        // epilogue: warp w reads tensor-memory lanes 32 (w % 4) .. (query
        // rows) and columns 64 (w / 4) .. of each tile; its candidates are
        // ranked by |t|^2 - 2 q.t (the row's |q|^2 is common to all)
        const int quarter = warp & 3, half = warp >> 2, etid = warp * 32 + lane;
        const int r = quarter * 32 + lane;
        const uint32_t row = q0 + (uint32_t)r;
        float c0 = INFINITY, c1 = INFINITY, c2 = INFINITY, c3 = INFINITY;
        int k0 = -1, k1 = -1, k2 = -1, k3 = -1;
        bool ok = true;
        for (int j = 0; j < ntile; ++j) {
            const int b = j & 1;
            const uint32_t col0 = (tile_lo + j) * kUN;
            // the tile's train norms (padded with +inf past the end); the
            // buffer of tile j was last read two tiles ago, before the barrier
            // of the tile in between
            if (etid < kUN) tnb[b * kUN + etid] = tn[col0 + etid];
            if (ok) ok = mbar_wait(acc_full + b, (j >> 1) & 1);
            epi_barrier();
            if (ok) {
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const float* tb = tnb + b * kUN + half * 64;
#pragma unroll 1
                for (int c = 0; c < 2; ++c) {
                    float v[32];
                    tmem_ld32(tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(b * kUN + half * 64 + 32 * c), v);
#pragma unroll
                    for (int i = 0; i < 32; ++i) {
                        const float d = fmaf(-2.0f, v[i], tb[32 * c + i]);
                        // columns rise, so a tie never goes before an earlier one
                        if (d < c3) {
                            const int col = (int)col0 + half * 64 + 32 * c + i;
                            const bool b0 = d < c0, b1 = d < c1, b2 = d < c2;
                            c3 = b2 ? c2 : d;
                            k3 = b2 ? k2 : col;
                            c2 = b1 ? c1 : (b2 ? d : c2);
                            k2 = b1 ? k1 : (b2 ? col : k2);
                            c1 = b0 ? c0 : (b1 ? d : c1);
                            k1 = b0 ? k0 : (b1 ? col : k1);
                            c0 = b0 ? d : c0;
                            k0 = b0 ? col : k0;
                        }
                    }
                }
                asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            } else {
                atomicOr(bad, 1u);
            }
            mbar_arrive(acc_empty + b);
        }
        // the second half's candidates to the first, then the exact
        // re-ranking of the union (the dot product as an FMA chain in index
        // order; ties to the lower train index)
        if (half == 1) {
            mrg_d[r * 4 + 0] = c0; mrg_i[r * 4 + 0] = k0;
            mrg_d[r * 4 + 1] = c1; mrg_i[r * 4 + 1] = k1;
            mrg_d[r * 4 + 2] = c2; mrg_i[r * 4 + 2] = k2;
            mrg_d[r * 4 + 3] = c3; mrg_i[r * 4 + 3] = k3;
        }
        epi_barrier();
        if (half == 0 && ok && row < nq) {
            // the 4 best of the 8 by (d, index): two sorted lists of 4
            int ci[kCand];
            {
                float da[8] = {c0, c1, c2, c3, mrg_d[r * 4], mrg_d[r * 4 + 1], mrg_d[r * 4 + 2], mrg_d[r * 4 + 3]};
                int ia[8] = {k0, k1, k2, k3, mrg_i[r * 4], mrg_i[r * 4 + 1], mrg_i[r * 4 + 2], mrg_i[r * 4 + 3]};
                int pa = 0, pb = 4;
#pragma unroll
                for (int k = 0; k < kCand; ++k) {
                    const bool takea = pb >= 8 || (pa < 4 && before(da[pa], ia[pa] < 0 ? 0x7fffffff : ia[pa], da[pb],
                                                                     ia[pb] < 0 ? 0x7fffffff : ia[pb]));
                    ci[k] = takea ? ia[pa] : ia[pb];
                    pa += takea ? 1 : 0;
                    pb += takea ? 0 : 1;
                }
            }
            const float qnr = qn[row];
            const float4* qv = reinterpret_cast<const float4*>(q + (size_t)row * kD);
            Best2 bst{INFINITY, INFINITY, -1, -1};
#pragma unroll 1
            for (int k = 0; k < kCand; ++k) {
                const int cj = ci[k];
                if (cj < 0) continue;
                const float4* tv = reinterpret_cast<const float4*>(t + (size_t)cj * kD);
                float dot = 0.0f;
#pragma unroll 8
                for (int k4 = 0; k4 < kD / 4; ++k4) {
                    const float4 a4 = qv[k4], c4 = tv[k4];
                    dot = fmaf(a4.x, c4.x, dot);
                    dot = fmaf(a4.y, c4.y, dot);
                    dot = fmaf(a4.z, c4.z, dot);
                    dot = fmaf(a4.w, c4.w, dot);
                }
                push(bst, fmaf(-2.0f, dot, qnr + tn[cj]), cj);
            }
            part[(size_t)chunk * nq + row] = make_float4(bst.d1, __int_as_float(bst.i1), bst.d2, __int_as_float(bst.i2));
        }
    }
    // every tensor-core operation of this CTA is complete before the barrier:
    // the epilogue waited for the last accumulator (or the MMA thread stopped)
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (*bad && tid == 0) atomicOr(err, 1u);
    if (warp == 9) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kUTmemCols) : "memory");
    }
}

// Fold the chunks of each query in chunk order and convert to distances.
__global__ void k_match_fold(const float4* __restrict__ part, uint32_t nq, uint32_t splits,
                             SiftCudaMatch* __restrict__ out, const uint32_t* __restrict__ err) {
    const uint32_t qi = blockIdx.x * blockDim.x + threadIdx.x;
    if (qi >= nq) return;
    Best2 b{INFINITY, INFINITY, -1, -1};
    for (uint32_t s = 0; s < splits && !*err; ++s) {
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

size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }
// train norms, padded to whole 128-descriptor tiles
size_t tn_floats(uint32_t nt) { return ((size_t)nt + 127) / 128 * 128; }

// Chunks of the train set for the tcgen05 kernel: enough (query tile, chunk)
// items for two CTAs per multiprocessor, at most 64 chunks.
void umma_chunks(uint32_t nq, uint32_t nt, uint32_t* chunk_tiles, uint32_t* n_chunks) {
    const uint32_t tt = (nt + kUN - 1) / kUN, qt = std::max<uint32_t>((nq + kUM - 1) / kUM, 1u);
    if (tt == 0) {
        *chunk_tiles = 0;
        *n_chunks = 0;
        return;
    }
    uint32_t want = std::min<uint32_t>(std::min<uint32_t>((2u * 152u + qt - 1) / qt, tt), 64u);
    *chunk_tiles = (tt + want - 1) / want;
    *n_chunks = (tt + *chunk_tiles - 1) / *chunk_tiles;
}

// Rows x 128 floats, boxes of 32 floats (128 bytes, the swizzle span) x 128
// rows; rows past the end read as zeros.
bool descriptor_map(CUtensorMap* m, const float* base, uint32_t rows) {
    EncodeTiledFn enc = encode_tiled();
    if (!enc) return false;
    const cuuint64_t dims[2] = {(cuuint64_t)kD, (cuuint64_t)rows};
    const cuuint64_t strides[1] = {(cuuint64_t)kD * sizeof(float)};
    const cuuint32_t box[2] = {32u, 128u};
    const cuuint32_t estr[2] = {1u, 1u};
    return enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float*>(base), dims, strides, box, estr,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace

size_t match_scratch_bytes(uint32_t nq, uint32_t nt) {
    uint32_t ct, nc;
    umma_chunks(nq, nt, &ct, &nc);
    return align256((size_t)nq * 4) + align256(tn_floats(nt) * 4) + 256 + (size_t)std::max<uint32_t>(nc, 1) * nq * sizeof(float4);
}

int launch_match(const float* d_q, uint32_t nq, const float* d_t, uint32_t nt, SiftCudaMatch* d_out, void* scratch,
                 cudaStream_t st) {
    if (nq == 0) return 0;
    uint32_t chunk_tiles, n_chunks;
    umma_chunks(nq, nt, &chunk_tiles, &n_chunks);
    char* p = static_cast<char*>(scratch);
    float* qn = reinterpret_cast<float*>(p);
    p += align256((size_t)nq * 4);
    float* tn = reinterpret_cast<float*>(p);
    p += align256(tn_floats(nt) * 4);
    uint32_t* err = reinterpret_cast<uint32_t*>(p);  // set by a tensor-core CTA whose wait ran out
    float4* part = reinterpret_cast<float4*>(p + 256);
    if (cudaMemsetAsync(err, 0, sizeof(uint32_t), st) != cudaSuccess) return -1;
    k_sq_norms<<<(nq + 255) / 256, 256, 0, st>>>(d_q, nq, qn, nq);
    if (n_chunks) {
        const uint32_t ntp = (uint32_t)tn_floats(nt);
        k_sq_norms<<<(ntp + 255) / 256, 256, 0, st>>>(d_t, nt, tn, ntp);
        CUtensorMap mq, mt;
        if (!descriptor_map(&mq, d_q, nq) || !descriptor_map(&mt, d_t, nt)) return -1;
        if (cudaFuncSetAttribute(k_match_umma, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kUSmem) != cudaSuccess)
            return -1;
        const uint32_t grid = ((nq + kUM - 1) / kUM) * n_chunks;
        k_match_umma<<<grid, kUThreads, kUSmem, st>>>(mq, mt, d_q, qn, nq, d_t, tn, nt, chunk_tiles, n_chunks, part,
                                                      err);
    }
    k_match_fold<<<(nq + 255) / 256, 256, 0, st>>>(part, nq, n_chunks, d_out, err);
    return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
}

// The error word of the last launch_match on this scratch (after it ran).
const uint32_t* match_error_word(const void* scratch, uint32_t nq, uint32_t nt) {
    return reinterpret_cast<const uint32_t*>(static_cast<const char*>(scratch) + align256((size_t)nq * 4) +
                                             align256(tn_floats(nt) * 4));
}

}  // namespace sift
