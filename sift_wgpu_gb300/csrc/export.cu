// export.cu — results of a finished run written straight into mapped pinned
// host memory by the device.
//
// The host does not know the keypoint count of a run before it finishes, so a
// copy engine cannot be told how much to move; this kernel reads the count on
// the device and moves the counters, min(count, cap) keypoints and their
// descriptors over the host link in one launch at the end of the run. The
// host then needs one synchronisation per call instead of a counter read
// followed by a sized copy.
#include "sift_internal.cuh"

namespace sift {
namespace {

__global__ void __launch_bounds__(256) k_export(const Counters* __restrict__ ctr, const Keypoint* __restrict__ kps,
                                                const float* __restrict__ desc, Counters* hctr, Keypoint* hkps,
                                                float* hdesc, uint32_t cap, int with_desc) {
    const uint32_t n = min(ctr->n_oriented, cap);
    const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x, stride = gridDim.x * blockDim.x;
    constexpr uint32_t kCtrWords = sizeof(Counters) / 4;
    if (tid < kCtrWords) reinterpret_cast<uint32_t*>(hctr)[tid] = reinterpret_cast<const uint32_t*>(ctr)[tid];
    const uint32_t kw = n * (uint32_t)(sizeof(Keypoint) / 4);
    for (uint32_t i = tid; i < kw; i += stride)
        reinterpret_cast<uint32_t*>(hkps)[i] = reinterpret_cast<const uint32_t*>(kps)[i];
    if (!with_desc) return;
    const uint32_t dv = n * (kDescLen / 4);
    for (uint32_t i = tid; i < dv; i += stride)
        reinterpret_cast<float4*>(hdesc)[i] = reinterpret_cast<const float4*>(desc)[i];
}

}  // namespace

int launch_export(const Counters* ctr, const Keypoint* kps, const float* desc, Counters* hctr, Keypoint* hkps,
                  float* hdesc, uint32_t cap, int with_desc, cudaStream_t st) {
    k_export<<<152 * 2, 256, 0, st>>>(ctr, kps, desc, hctr, hkps, hdesc, cap, with_desc);
    return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace sift
