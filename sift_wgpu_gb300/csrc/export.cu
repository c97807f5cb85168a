// export.cu — counters and keypoints of a finished run written straight into
// mapped pinned host memory by the device.
//
// The host does not know the keypoint count of a run before it finishes, so a
// copy engine cannot be told how much to move; this kernel reads the count on
// the device and moves the counters and min(count, cap) keypoints over the
// host link in one launch at the end of the run. (The descriptor stage of such
// a run writes descriptors below cap into the same buffer itself, describe.cu.)
// The host then needs one synchronisation per call instead of a counter read
// followed by a sized copy.
#include "sift_internal.cuh"

namespace sift {
namespace {

__global__ void __launch_bounds__(256) k_export(const Counters* __restrict__ ctr, const Keypoint* __restrict__ kps,
                                                Counters* hctr, Keypoint* hkps, uint32_t cap) {
    chain_wait();
    const uint32_t n = min(ctr->n_oriented, cap);
    const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x, stride = gridDim.x * blockDim.x;
    constexpr uint32_t kCtrWords = sizeof(Counters) / 4;
    if (tid < kCtrWords) reinterpret_cast<uint32_t*>(hctr)[tid] = reinterpret_cast<const uint32_t*>(ctr)[tid];
    const size_t kw = (size_t)n * (sizeof(Keypoint) / 4);
    for (size_t i = tid; i < kw; i += stride)
        reinterpret_cast<uint32_t*>(hkps)[i] = reinterpret_cast<const uint32_t*>(kps)[i];
}

}  // namespace

int launch_export(const Counters* ctr, const Keypoint* kps, Counters* hctr, Keypoint* hkps, uint32_t cap,
                  cudaStream_t st) {
    if (launch_chained(k_export, 152, 256, 0, st, ctr, kps, hctr, hkps, cap) != cudaSuccess)
        return -1;
    return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace sift
