// scan.cu — deterministic exclusive prefix sum used for ordered compaction.
//
// Three launches (tile reduce, scan of tile sums, tile scan) with a fixed
// tile order, so every output position is a pure function of the inputs. The
// element count may live in device memory (n_dev) so that a stage whose
// length is only known on the GPU needs no host round trip; the grid is then
// sized for the host bound and surplus tiles exit.
#include "sift_internal.cuh"

namespace sift {
namespace {

constexpr int kThreads = 256;
constexpr int kItems = 8;
constexpr int kTile = kThreads * kItems;

template <int MODE>
__device__ __forceinline__ uint32_t load_item(const uint32_t* in, size_t i, size_t n) {
    if (i >= n) return 0u;
    uint32_t v = in[i];
    return MODE == SCAN_POPC ? (uint32_t)__popc(v) : v;
}

__device__ __forceinline__ size_t eff_n(size_t n, const uint32_t* n_dev) {
    if (n_dev) {
        size_t d = *n_dev;
        return d < n ? d : n;
    }
    return n;
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

template <int MODE>
__global__ void __launch_bounds__(kThreads) k_scan_reduce(const uint32_t* __restrict__ in, size_t n,
                                                          const uint32_t* __restrict__ n_dev,
                                                          uint32_t* __restrict__ partials) {
    const size_t N = eff_n(n, n_dev);
    const size_t base = (size_t)blockIdx.x * kTile;
    if (base >= N) {
        if (threadIdx.x == 0) partials[blockIdx.x] = 0u;
        return;
    }
    uint32_t s = 0;
#pragma unroll
    for (int k = 0; k < kItems; ++k) s += load_item<MODE>(in, base + (size_t)k * kThreads + threadIdx.x, N);
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) s += __shfl_xor_sync(0xffffffffu, s, d);
    __shared__ uint32_t ws[kThreads / 32];
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t t = 0;
        for (int w = 0; w < kThreads / 32; ++w) t += ws[w];
        partials[blockIdx.x] = t;
    }
}

// One CTA scans the tile sums in place (exclusive) and writes the total.
__global__ void __launch_bounds__(kThreads) k_scan_partials(uint32_t* __restrict__ partials, size_t nb,
                                                            uint32_t* __restrict__ total_out) {
    __shared__ uint32_t carry_s;
    __shared__ uint32_t chunk_total;
    if (threadIdx.x == 0) carry_s = 0u;
    __syncthreads();
    for (size_t base = 0; base < nb; base += kThreads) {
        size_t i = base + threadIdx.x;
        uint32_t v = i < nb ? partials[i] : 0u;
        uint32_t ex = block_exclusive(v, &chunk_total);
        uint32_t carry = carry_s;
        if (i < nb) partials[i] = carry + ex;
        __syncthreads();
        if (threadIdx.x == 0) carry_s = carry + chunk_total;
        __syncthreads();
    }
    if (threadIdx.x == 0 && total_out) *total_out = carry_s;
}

template <int MODE>
__global__ void __launch_bounds__(kThreads) k_scan_down(const uint32_t* __restrict__ in,
                                                        uint32_t* __restrict__ out, size_t n,
                                                        const uint32_t* __restrict__ n_dev,
                                                        const uint32_t* __restrict__ partials) {
    const size_t N = eff_n(n, n_dev);
    const size_t base = (size_t)blockIdx.x * kTile;
    if (base >= N) return;
    // Each thread owns kItems consecutive elements.
    const size_t mine = base + (size_t)threadIdx.x * kItems;
    uint32_t v[kItems];
    uint32_t s = 0;
#pragma unroll
    for (int k = 0; k < kItems; ++k) {
        v[k] = load_item<MODE>(in, mine + k, N);
        s += v[k];
    }
    __shared__ uint32_t tot;
    uint32_t ex = block_exclusive(s, &tot) + partials[blockIdx.x];
#pragma unroll
    for (int k = 0; k < kItems; ++k) {
        if (mine + k < N) out[mine + k] = ex;
        ex += v[k];
    }
}

}  // namespace

size_t scan_partials_size(size_t n) { return (n + kTile - 1) / kTile + 1; }

int scan_launches(size_t) { return 3; }

int scan_exclusive(const uint32_t* in, ScanInput mode, uint32_t* out, size_t n, const uint32_t* n_dev,
                   uint32_t* total_out, uint32_t* partials, cudaStream_t st) {
    if (n == 0) {
        if (total_out) cudaMemsetAsync(total_out, 0, sizeof(uint32_t), st);
        return 0;
    }
    const size_t nb = (n + kTile - 1) / kTile;
    if (mode == SCAN_POPC) {
        k_scan_reduce<SCAN_POPC><<<(unsigned)nb, kThreads, 0, st>>>(in, n, n_dev, partials);
    } else {
        k_scan_reduce<SCAN_U32><<<(unsigned)nb, kThreads, 0, st>>>(in, n, n_dev, partials);
    }
    k_scan_partials<<<1, kThreads, 0, st>>>(partials, nb, total_out);
    if (mode == SCAN_POPC) {
        k_scan_down<SCAN_POPC><<<(unsigned)nb, kThreads, 0, st>>>(in, out, n, n_dev, partials);
    } else {
        k_scan_down<SCAN_U32><<<(unsigned)nb, kThreads, 0, st>>>(in, out, n, n_dev, partials);
    }
    return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace sift
