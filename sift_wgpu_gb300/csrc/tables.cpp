// tables.cpp — host-side filter tables of the pyramid.
//
// The blur kernels and the Lanczos3 resampling taps depend only on the
// parameters and the image size, so they are built once on the host (in f32,
// the way the reference builds them) and uploaded; every GPU thread then uses
// the identical weights. Compiled with -ffp-contract=off so that each product
// and sum is rounded separately, as in Rust.
//
//  * gaussian_kernel: imageproc 0.25.0 gaussian_blur_f32's kernel (the crate
//    is a dependency of the reference, Cargo.lock:648-650, not vendored):
//    radius ceil(2 sigma), taps (sqrt(2 pi) sigma)^-1 exp(-x^2 / (2 sigma^2)).
//  * lanczos_axis: image 0.25.6 resize's per-axis taps (Cargo.lock:634-636):
//    centre (i + 0.5) * ratio, support 3 * max(ratio, 1), window clamped to
//    the source, lanczos3((j - centre + 0.5) / max(ratio, 1)) normalised by
//    the window's sum.
//  * blur_sigmas: the increments of generate_gaussian_pyramid
//    (src/sift.rs:129-177) and the base blur (src/sift.rs:1204-1214).
#include "tables.h"

#include <algorithm>
#include <cmath>

namespace sift {

namespace {
constexpr float kPiF = 3.14159265358979323846f;

// f32::powi with a run-time exponent (repeated squaring, as compiler
// builtins evaluate it).
float powi(float a, int b) {
    bool recip = b < 0;
    unsigned n = recip ? 0u - (unsigned)b : (unsigned)b;
    float r = 1.0f;
    for (;;) {
        if (n & 1u) r *= a;
        n >>= 1;
        if (n == 0) break;
        a *= a;
    }
    return recip ? 1.0f / r : r;
}

float sinc(float t) {
    float a = t * kPiF;
    if (t == 0.0f) return 1.0f;
    return std::sin(a) / a;
}

float lanczos3(float x) {
    if (std::fabs(x) < 3.0f) return sinc(x) * sinc(x / 3.0f);
    return 0.0f;
}
}  // namespace

std::vector<float> gaussian_kernel(float sigma) {
    float fr = std::ceil(2.0f * sigma);
    int radius = fr > 0.0f ? (int)fr : 0;
    std::vector<float> k((size_t)(2 * radius + 1), 0.0f);
    float c = 1.0f / (std::sqrt(2.0f * kPiF) * sigma);
    for (int i = 0; i <= radius; ++i) {
        float x = (float)i;
        float v = c * std::exp(-(x * x) / (2.0f * (sigma * sigma)));
        k[(size_t)(radius + i)] = v;
        k[(size_t)(radius - i)] = v;
    }
    return k;
}

AxisTaps lanczos_axis(uint32_t src, uint32_t dst) {
    AxisTaps t;
    float ratio = (float)src / (float)dst;
    float sratio = ratio < 1.0f ? 1.0f : ratio;
    float support = 3.0f * sratio;
    for (uint32_t o = 0; o < dst; ++o) {
        float input = ((float)o + 0.5f) * ratio;
        long long left = (long long)std::floor(input - support);
        left = std::max<long long>(0, std::min<long long>(left, (long long)src - 1));
        long long right = (long long)std::ceil(input + support);
        right = std::max<long long>(left + 1, std::min<long long>(right, (long long)src));
        input = input - 0.5f;
        t.left.push_back((int)left);
        t.count.push_back((int)(right - left));
        t.woff.push_back((int)t.w.size());
        size_t base = t.w.size();
        float sum = 0.0f;
        for (long long i = left; i < right; ++i) {
            float wv = lanczos3(((float)i - input) / sratio);
            t.w.push_back(wv);
            sum += wv;
        }
        for (size_t j = base; j < t.w.size(); ++j) t.w[j] /= sum;
    }
    return t;
}

BlurPlan blur_plan(const SiftCudaParams& p) {
    BlurPlan b;
    b.base = p.sigma > p.assumed_blur ? std::sqrt(p.sigma * p.sigma - p.assumed_blur * p.assumed_blur) : 0.0f;
    if (!(b.base > 1e-4f)) b.base = 0.0f;
    float k = std::pow(2.0f, 1.0f / (float)p.num_intervals);
    std::vector<float> target;
    for (uint32_t s = 0; s < p.num_intervals + 3; ++s) target.push_back(p.sigma * powi(k, (int)s));
    for (uint32_t o = 0; o < p.num_octaves; ++o) {
        float scale = std::ldexp(1.0f, (int)o);
        float prev = p.sigma * scale;
        std::vector<float> row;
        for (uint32_t s = 1; s < p.num_intervals + 3; ++s) {
            float t = target[s] * scale;
            float blur = std::sqrt(t * t - prev * prev);
            row.push_back(blur < 1e-4f ? 0.0f : blur);
            prev = t;
        }
        b.level.push_back(row);
    }
    return b;
}

}  // namespace sift
