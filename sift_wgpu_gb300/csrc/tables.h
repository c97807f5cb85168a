// tables.h — host-side filter tables (tables.cpp).
#pragma once

#include <stdint.h>

#include <vector>

#include "../../include/sift_cuda.h"

namespace sift {

struct AxisTaps {
    std::vector<int> left, count, woff;
    std::vector<float> w;
};

struct BlurPlan {
    float base;                             // base blur sigma, 0 = none
    std::vector<std::vector<float>> level;  // [octave][s-1], 0 = copy level
};

std::vector<float> gaussian_kernel(float sigma);
AxisTaps lanczos_axis(uint32_t src, uint32_t dst);
BlurPlan blur_plan(const SiftCudaParams& p);

}  // namespace sift
