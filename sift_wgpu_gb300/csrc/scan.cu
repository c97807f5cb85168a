// scan.cu — deterministic exclusive prefix sum used for ordered compaction.
//
// One launch per scan (single pass with decoupled look-back): each CTA takes
// the next tile ticket, reduces its tile, publishes the tile sum, then walks
// back over its predecessors' published sums until it meets an inclusive
// prefix, publishes its own inclusive prefix and writes its outputs. A CTA
// waits only on tiles whose tickets were handed out before its own, to CTAs
// already running, so every wait ends; each wait is bounded anyway, and a
// wait that runs out sets bit 8 of the run's overflow word instead of
// hanging. Every output is an exact integer sum, so the result does not
// depend on scheduling.
//
// The element count may live in device memory (n_dev) so that a stage whose
// length is only known on the GPU needs no host round trip; the grid is then
// sized for the host bound and tiles past the end exit at once.
//
// State: scan_state_words(n) 64-bit words per scan — a ticket counter and one
// status word per tile (flag << 32 | value; flag 1 = tile sum, 2 = inclusive
// prefix), zero before the scan runs.
#include "sift_internal.cuh"

namespace sift {
namespace {

constexpr int kThreads = 256;
constexpr int kItems = 8;
constexpr int kTile = kThreads * kItems;
constexpr unsigned kMaxWaits = 1u << 20;  // x ~64 ns: a wait gives up after ~0.1 s

template <int MODE>
__device__ __forceinline__ uint32_t load_item(const uint32_t* in, size_t i, size_t n) {
    if (i >= n) return 0u;
    uint32_t v = in[i];
    return MODE == SCAN_POPC ? (uint32_t)__popc(v) : v;
}

// Block-wide exclusive scan of one value per thread; returns the exclusive
// prefix and writes the block total to *total.
__device__ __forceinline__ uint32_t block_exclusive(uint32_t v, uint32_t* total) {
    __shared__ uint32_t warp_sums[kThreads / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, d);
        if (lane >= d) x += y;
    }
    if (lane == 31) warp_sums[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = lane < kThreads / 32 ? warp_sums[lane] : 0u;
        uint32_t s = w;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, s, d);
            if (lane >= d) s += y;
        }
        if (lane < kThreads / 32) warp_sums[lane] = s - w;  // exclusive
        if (lane == kThreads / 32 - 1) *total = s;
    }
    __syncthreads();
    uint32_t r = x - v + warp_sums[warp];
    __syncthreads();
    return r;
}

__device__ __forceinline__ void publish(unsigned long long* slot, unsigned long long flag, uint32_t v) {
    __threadfence();
    atomicExch(slot, (flag << 32) | v);
}

template <int MODE>
__global__ void __launch_bounds__(kThreads) k_scan(const uint32_t* __restrict__ in, uint32_t* __restrict__ out,
                                                   size_t n, const uint32_t* __restrict__ n_dev,
                                                   uint32_t* __restrict__ total_out,
                                                   unsigned long long* __restrict__ state, uint32_t* err) {
    chain_wait();
    __shared__ uint32_t s_tile, s_excl, s_tot;
    if (threadIdx.x == 0) s_tile = atomicAdd(reinterpret_cast<unsigned int*>(state), 1u);
    __syncthreads();
    const uint32_t tile = s_tile;
    size_t N = n;
    if (n_dev) {
        const size_t d = *n_dev;
        N = d < n ? d : n;
    }
    const size_t base = (size_t)tile * kTile;
    if (base >= N && tile != 0) return;  // no later tile waits on this one
    // each thread owns kItems consecutive elements
    const size_t mine = base + (size_t)threadIdx.x * kItems;
    uint32_t v[kItems];
    uint32_t s = 0;
#pragma unroll
    for (int k = 0; k < kItems; ++k) {
        v[k] = load_item<MODE>(in, mine + k, N);
        s += v[k];
    }
    uint32_t ex = block_exclusive(s, &s_tot);
    if (threadIdx.x == 0) {
        unsigned long long* st = state + 1;
        const uint32_t tot = s_tot;
        uint32_t excl = 0;
        if (tile == 0) {
            publish(st, 2ull, tot);
        } else {
            publish(st + tile, 1ull, tot);
            for (int p = (int)tile - 1; p >= 0; --p) {
                unsigned long long w = 0;
                unsigned waits = 0;
                while ((w = *reinterpret_cast<volatile unsigned long long*>(st + p)) >> 32 == 0ull &&
                       ++waits < kMaxWaits)
                    __nanosleep(64);
                if (w >> 32 == 0ull) {
                    atomicOr(err, 8u);  // gave up: the outputs of this scan are wrong, the run reports it
                    break;
                }
                excl += (uint32_t)w;
                if (w >> 32 == 2ull) break;
            }
            publish(st + tile, 2ull, excl + tot);
        }
        s_excl = excl;
        if (total_out && base + kTile >= N) *total_out = excl + tot;  // the tile holding the last element
    }
    __syncthreads();
    ex += s_excl;
#pragma unroll
    for (int k = 0; k < kItems; ++k) {
        if (mine + k < N) out[mine + k] = ex;
        ex += v[k];
    }
}

}  // namespace

size_t scan_state_words(size_t n) { return (n + kTile - 1) / kTile + 1; }

int scan_exclusive(const uint32_t* in, ScanInput mode, uint32_t* out, size_t n, const uint32_t* n_dev,
                   uint32_t* total_out, unsigned long long* state, uint32_t* err, cudaStream_t st) {
    if (n == 0) {
        if (total_out) cudaMemsetAsync(total_out, 0, sizeof(uint32_t), st);
        return 0;
    }
    const unsigned nb = (unsigned)((n + kTile - 1) / kTile);
    const cudaError_t e =
        mode == SCAN_POPC
            ? launch_chained(k_scan<SCAN_POPC>, nb, kThreads, 0, st, in, out, n, n_dev, total_out, state, err)
            : launch_chained(k_scan<SCAN_U32>, nb, kThreads, 0, st, in, out, n, n_dev, total_out, state, err);
    if (e != cudaSuccess) return -1;
    return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace sift
