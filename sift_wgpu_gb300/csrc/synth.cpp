// synth.cpp — seeded synthetic grayscale images.
//
// The benchmark images of this engine: background 128, isotropic Gaussian
// blobs, filled rectangles drawn over them, i.i.d. N(0, 3^2) noise, clamped
// and rounded to u8. The RNG is xoshiro256** seeded through splitmix64
// (Blackman & Vigna), normals by Box-Muller; everything in f64 so the same
// seed gives the same image on any host.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "../../include/sift_cuda.h"

namespace {

struct Xoshiro256ss {
    uint64_t s[4];
    static uint64_t splitmix64(uint64_t& x) {
        uint64_t z = (x += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    explicit Xoshiro256ss(uint64_t seed) {
        uint64_t x = seed;
        for (auto& v : s) v = splitmix64(x);
    }
    static uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
    uint64_t next() {
        const uint64_t result = rotl(s[1] * 5, 7) * 9;
        const uint64_t t = s[1] << 17;
        s[2] ^= s[0];
        s[3] ^= s[1];
        s[1] ^= s[2];
        s[0] ^= s[3];
        s[2] ^= t;
        s[3] = rotl(s[3], 45);
        return result;
    }
    double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }  // [0, 1)
    double normal() {
        double u1 = 1.0 - uniform();  // (0, 1]
        double u2 = uniform();
        return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
    }
};

}  // namespace

extern "C" void sift_synth_density(uint32_t width, uint32_t height, uint32_t* n_blobs, uint32_t* n_rects) {
    double area = (double)width * (double)height / (512.0 * 512.0);
    if (n_blobs) *n_blobs = (uint32_t)std::llround(200.0 * area);
    if (n_rects) *n_rects = (uint32_t)std::llround(40.0 * area);
}

extern "C" void sift_synth_image(uint64_t seed, uint32_t width, uint32_t height, uint32_t n_blobs,
                                 uint32_t n_rects, uint8_t* out) {
    if (!out || width == 0 || height == 0) return;
    const int W = (int)width, H = (int)height;
    std::vector<double> img((size_t)W * H, 128.0);
    Xoshiro256ss rng(seed);
    for (uint32_t b = 0; b < n_blobs; ++b) {
        double cx = rng.uniform() * W, cy = rng.uniform() * H;
        double sg = 2.0 + 18.0 * rng.uniform();
        double amp = -90.0 + 180.0 * rng.uniform();
        int rad = (int)std::ceil(4.0 * sg);
        int x0 = std::max(0, (int)std::floor(cx) - rad), x1 = std::min(W - 1, (int)std::floor(cx) + rad);
        int y0 = std::max(0, (int)std::floor(cy) - rad), y1 = std::min(H - 1, (int)std::floor(cy) + rad);
        double inv = 1.0 / (2.0 * sg * sg);
        for (int y = y0; y <= y1; ++y) {
            double dy = (double)y - cy;
            for (int x = x0; x <= x1; ++x) {
                double dx = (double)x - cx;
                img[(size_t)y * W + x] += amp * std::exp(-(dx * dx + dy * dy) * inv);
            }
        }
    }
    for (uint32_t r = 0; r < n_rects; ++r) {
        int rx = (int)(rng.uniform() * W), ry = (int)(rng.uniform() * H);
        int rw = 8 + (int)(rng.uniform() * 89.0), rh = 8 + (int)(rng.uniform() * 89.0);
        double v = std::floor(rng.uniform() * 256.0);
        for (int y = ry; y < std::min(H, ry + rh); ++y)
            for (int x = rx; x < std::min(W, rx + rw); ++x) img[(size_t)y * W + x] = v;
    }
    for (size_t i = 0; i < img.size(); ++i) {
        double v = img[i] + 3.0 * rng.normal();
        v = v < 0.0 ? 0.0 : (v > 255.0 ? 255.0 : v);
        out[i] = (uint8_t)std::lround(v);
    }
}
