// sift_oracle.cpp — CPU restatement of the reference CPU SIFT path.
//
// TEST INFRASTRUCTURE ONLY: the checker for the CUDA path and the timed CPU
// baseline. Every function cites the reference file:line it restates
// (src/sift.rs of stevel705/sift-wgpu unless stated otherwise). f32 operations
// are written in the reference's order; build with -ffp-contract=off so no
// multiply-add is fused (Rust never contracts). Rust's f32 transcendental calls
// go to the platform libm on Linux, so expf/atan2f/sinf/cosf/powf/sqrtf are
// called here the same way.
//
// Third-party arithmetic (not vendored in the reference; parity unpinned):
//  * imageproc 0.25.0 gaussian_blur_f32 (Cargo.lock:648-650): kernel radius
//    ceil(2 sigma), samples of the Gaussian density, separable horizontal then
//    vertical correlation with clamp-to-edge, f32 accumulation from 0 in tap
//    order, each pass stored back to u8 through imageproc's Clamp (truncation).
//  * image 0.25.6 resize_exact(Lanczos3) (Cargo.lock:634-636): vertical pass to
//    an f32 intermediate, then horizontal pass; Lanczos-3 windowed sinc with the
//    support scaled by the downscale ratio, weights normalised per output pixel,
//    f32 accumulation, final clamp to [0,255] and round-to-nearest.
#include "sift_oracle.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <thread>
#include <vector>

namespace {

constexpr float kPi = 3.14159265358979323846f;  // f32::consts::PI
constexpr int kMaxInterpSteps = 5;               // src/sift.rs:18
constexpr float kInterpOffsetThr = 0.5f;         // src/sift.rs:19
constexpr int kOriBins = 36;                     // src/sift.rs:21
constexpr float kOriRadiusFactor = 3.0f;         // src/sift.rs:22
constexpr int kOriSmoothIters = 2;               // src/sift.rs:23
constexpr float kOriPeakRatio = 0.8f;            // src/sift.rs:24
constexpr float kOriSigmaFactor = 1.5f;          // src/sift.rs:25
constexpr int kDescBins = 8;                     // src/sift.rs:28
constexpr int kDescWidth = 4;                    // src/sift.rs:29
constexpr float kDescMagThr = 0.2f;              // src/sift.rs:30
constexpr float kDescPatchScale = 3.0f;          // src/sift.rs:31
constexpr int kDescLen = kDescWidth * kDescWidth * kDescBins;

OracleBlurModel g_blur_model = {200, 0, 0};

// ---- Rust scalar semantics -------------------------------------------------

// `f as i32`: saturating, NaN -> 0.
inline int32_t as_i32(float v) {
    if (std::isnan(v)) return 0;
    if (v >= 2147483648.0f) return INT32_MAX;
    if (v <= -2147483648.0f) return INT32_MIN;
    return (int32_t)v;
}
// `f as usize`: saturating at 0, NaN -> 0.
inline uint64_t as_usize(float v) {
    if (std::isnan(v) || v <= 0.0f) return 0;
    if (v >= 18446744073709551616.0f) return UINT64_MAX;
    return (uint64_t)v;
}
// f32::rem_euclid
inline float rem_euclid(float a, float b) {
    float r = std::fmod(a, b);
    return r < 0.0f ? r + std::fabs(b) : r;
}
// f32::powi with a run-time exponent (compiler_builtins __powisf2).
inline float powi(float a, int b) {
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
// 2.0_f32.powi(o) for the octave scale factors: an exact power of two.
inline float pow2i(int o) { return std::ldexp(1.0f, o); }

// ---- image containers --------------------------------------------------------

struct Gray {  // image::GrayImage
    uint32_t w = 0, h = 0;
    std::vector<uint8_t> px;
    Gray() = default;
    Gray(uint32_t w_, uint32_t h_) : w(w_), h(h_), px((size_t)w_ * h_, 0) {}
    uint8_t at(uint32_t x, uint32_t y) const { return px[(size_t)y * w + x]; }
};
struct ImgF {  // ImageBuffer<Luma<f32>, Vec<f32>>
    uint32_t w = 0, h = 0;
    std::vector<float> px;
    ImgF() = default;
    ImgF(uint32_t w_, uint32_t h_) : w(w_), h(h_), px((size_t)w_ * h_, 0.0f) {}
    float at(uint32_t x, uint32_t y) const { return px[(size_t)y * w + x]; }
};

// ---- a minimal rayon stand-in ------------------------------------------------

int g_threads = 1;

void parallel_for(size_t n, const std::function<void(size_t)>& fn) {
    int t = g_threads;
    if (t <= 1 || n < 2) {
        for (size_t i = 0; i < n; ++i) fn(i);
        return;
    }
    std::atomic<size_t> next{0};
    auto worker = [&]() {
        for (;;) {
            size_t i = next.fetch_add(1);
            if (i >= n) break;
            fn(i);
        }
    };
    int nt = (int)std::min<size_t>((size_t)t, n);
    std::vector<std::thread> pool;
    pool.reserve(nt - 1);
    for (int k = 1; k < nt; ++k) pool.emplace_back(worker);
    worker();
    for (auto& th : pool) th.join();
}

// ---- imageproc 0.25.0 gaussian_blur_f32 (restated; parity unpinned) -----------

// imageproc filter::gaussian: (sqrt(2 pi) * r).recip() * exp(-x^2 / (2 r^2)).
float gaussian_density(float x, float r) {
    float c = 1.0f / (std::sqrt(2.0f * kPi) * r);
    return c * std::exp(-(x * x) / (2.0f * (r * r)));
}

std::vector<float> gaussian_kernel(float sigma) {
    float f = (float)g_blur_model.blur_radius_factor_x100 / 100.0f;
    int radius = (int)as_usize(std::ceil(f * sigma));
    std::vector<float> k((size_t)(2 * radius + 1), 0.0f);
    for (int i = 0; i <= radius; ++i) {
        float v = gaussian_density((float)i, sigma);
        k[(size_t)(radius + i)] = v;
        k[(size_t)(radius - i)] = v;
    }
    if (g_blur_model.blur_normalize) {
        float s = 0.0f;
        for (float v : k) s += v;
        for (float& v : k) v /= s;
    }
    return k;
}

// imageproc Clamp<f32> for u8.
inline uint8_t clamp_u8(float a) {
    if (g_blur_model.blur_round) a = std::round(a);
    if (a < 255.0f) {
        if (a > 0.0f) return (uint8_t)a;
        return 0;
    }
    return 255;
}

Gray horizontal_filter(const Gray& in, const std::vector<float>& k) {
    Gray out(in.w, in.h);
    const int kw = (int)k.size(), half = kw / 2, W = (int)in.w;
    for (uint32_t y = 0; y < in.h; ++y) {
        const uint8_t* row = &in.px[(size_t)y * in.w];
        for (int x = 0; x < W; ++x) {
            float acc = 0.0f;
            for (int i = 0; i < kw; ++i) {
                int xs = std::max(0, std::min(x + i - half, W - 1));
                acc = acc + (float)row[xs] * k[(size_t)i];
            }
            out.px[(size_t)y * in.w + x] = clamp_u8(acc);
        }
    }
    return out;
}

Gray vertical_filter(const Gray& in, const std::vector<float>& k) {
    Gray out(in.w, in.h);
    const int kh = (int)k.size(), half = kh / 2, H = (int)in.h;
    for (int y = 0; y < H; ++y) {
        for (uint32_t x = 0; x < in.w; ++x) {
            float acc = 0.0f;
            for (int i = 0; i < kh; ++i) {
                int ys = std::max(0, std::min(y + i - half, H - 1));
                acc = acc + (float)in.px[(size_t)ys * in.w + x] * k[(size_t)i];
            }
            out.px[(size_t)y * in.w + x] = clamp_u8(acc);
        }
    }
    return out;
}

Gray gaussian_blur_f32(const Gray& in, float sigma) {
    auto k = gaussian_kernel(sigma);
    if (in.w == 0 || in.h == 0) return in;
    return vertical_filter(horizontal_filter(in, k), k);
}

// ---- image 0.25.6 resize_exact(Lanczos3) (restated; parity unpinned) ----------

float sinc(float t) {
    float a = t * kPi;
    if (t == 0.0f) return 1.0f;
    return std::sin(a) / a;
}
float lanczos3(float x) {
    const float t = 3.0f;
    if (std::fabs(x) < t) return sinc(x) * sinc(x / t);
    return 0.0f;
}

// One axis of the resampler: for each output index, [left, left+len) and the
// normalised weights.
struct AxisTaps {
    std::vector<uint32_t> left;
    std::vector<uint32_t> count;
    std::vector<float> w;  // concatenated
    std::vector<uint32_t> off;
};

AxisTaps lanczos_axis(uint32_t src, uint32_t dst) {
    AxisTaps t;
    float ratio = (float)src / (float)dst;
    float sratio = ratio < 1.0f ? 1.0f : ratio;
    float support = 3.0f * sratio;
    for (uint32_t o = 0; o < dst; ++o) {
        float input = ((float)o + 0.5f) * ratio;
        int64_t left = (int64_t)std::floor(input - support);
        left = std::max<int64_t>(0, std::min<int64_t>(left, (int64_t)src - 1));
        int64_t right = (int64_t)std::ceil(input + support);
        right = std::max<int64_t>(left + 1, std::min<int64_t>(right, (int64_t)src));
        input = input - 0.5f;
        t.left.push_back((uint32_t)left);
        t.count.push_back((uint32_t)(right - left));
        t.off.push_back((uint32_t)t.w.size());
        size_t base = t.w.size();
        float sum = 0.0f;
        for (int64_t i = left; i < right; ++i) {
            float wv = lanczos3(((float)i - input) / sratio);
            t.w.push_back(wv);
            sum += wv;
        }
        for (size_t j = base; j < t.w.size(); ++j) t.w[j] /= sum;
    }
    return t;
}

Gray resize_lanczos3(const Gray& in, uint32_t nw, uint32_t nh) {
    if (in.w == 0 || in.h == 0) return Gray(nw, nh);
    if (nw == in.w && nh == in.h) return in;
    // vertical_sample -> f32 intermediate of in.w x nh
    AxisTaps ty = lanczos_axis(in.h, nh);
    std::vector<float> tmp((size_t)in.w * nh, 0.0f);
    for (uint32_t oy = 0; oy < nh; ++oy) {
        for (uint32_t x = 0; x < in.w; ++x) {
            float t = 0.0f;
            for (uint32_t i = 0; i < ty.count[oy]; ++i)
                t += (float)in.at(x, ty.left[oy] + i) * ty.w[ty.off[oy] + i];
            tmp[(size_t)oy * in.w + x] = t;
        }
    }
    // horizontal_sample -> u8
    Gray out(nw, nh);
    if (nw == 0) return out;
    AxisTaps tx = lanczos_axis(in.w, nw);
    for (uint32_t ox = 0; ox < nw; ++ox) {
        for (uint32_t y = 0; y < nh; ++y) {
            float t = 0.0f;
            for (uint32_t i = 0; i < tx.count[ox]; ++i)
                t += tmp[(size_t)y * in.w + tx.left[ox] + i] * tx.w[tx.off[ox] + i];
            float c = t < 0.0f ? 0.0f : (t > 255.0f ? 255.0f : t);
            out.px[(size_t)y * nw + ox] = (uint8_t)std::round(c);
        }
    }
    return out;
}

// ---- src/sift.rs ------------------------------------------------------------

struct Sift {
    OracleParams p;

    // generate_gaussian_pyramid (src/sift.rs:129-177)
    std::vector<std::vector<Gray>> gaussian_pyramid(const Gray& base) const {
        std::vector<std::vector<Gray>> pyr;
        Gray cur = base;
        float k = std::pow(2.0f, 1.0f / (float)p.num_intervals);
        std::vector<float> target;
        for (uint32_t s = 0; s < p.num_intervals + 3; ++s) target.push_back(p.sigma * powi(k, (int)s));
        for (uint32_t o = 0; o < p.num_octaves; ++o) {
            std::vector<Gray> levels;
            levels.push_back(cur);
            float prev = p.sigma * pow2i((int)o);
            for (uint32_t s = 1; s < p.num_intervals + 3; ++s) {
                float t = target[s] * pow2i((int)o);
                float blur = std::sqrt(t * t - prev * prev);
                if (blur < 1e-4f)
                    levels.push_back(levels.back());
                else
                    levels.push_back(gaussian_blur_f32(levels.back(), blur));
                prev = t;
            }
            pyr.push_back(std::move(levels));
            if (o + 1 < p.num_octaves) {
                const Gray& src = pyr.back()[p.num_intervals];
                cur = resize_lanczos3(src, src.w / 2, src.h / 2);
            }
        }
        return pyr;
    }

    // generate_dog_pyramid (src/sift.rs:182-204) with convert_u8_to_f32_gray
    // (src/sift.rs:92-101) and subtract_f32_images (src/sift.rs:104-124).
    std::vector<std::vector<ImgF>> dog_pyramid(const std::vector<std::vector<Gray>>& g) const {
        std::vector<std::vector<ImgF>> dog(g.size());
        std::vector<std::pair<size_t, size_t>> jobs;
        for (size_t o = 0; o < g.size(); ++o) {
            dog[o].resize(g[o].size() - 1);
            for (size_t i = 0; i + 1 < g[o].size(); ++i) jobs.emplace_back(o, i);
        }
        parallel_for(jobs.size(), [&](size_t j) {
            size_t o = jobs[j].first, i = jobs[j].second;
            const Gray& a = g[o][i + 1];
            const Gray& b = g[o][i];
            ImgF d(a.w, a.h);
            for (size_t q = 0; q < a.px.size(); ++q)
                d.px[q] = (float)a.px[q] / 255.0f - (float)b.px[q] / 255.0f;
            dog[o][i] = std::move(d);
        });
        return dog;
    }

    // get_pixel_value (src/sift.rs:208-214)
    static float pix(const ImgF& im, int x, int y) {
        int xc = std::max(0, std::min(x, (int)im.w - 1));
        int yc = std::max(0, std::min(y, (int)im.h - 1));
        return im.at((uint32_t)xc, (uint32_t)yc);
    }
    // get_gauss_pixel_value (src/sift.rs:218-223)
    static float gpix(const Gray& im, int x, int y) {
        int xc = std::max(0, std::min(x, (int)im.w - 1));
        int yc = std::max(0, std::min(y, (int)im.h - 1));
        return (float)im.at((uint32_t)xc, (uint32_t)yc) / 255.0f;
    }

    // find_scale_space_extrema (src/sift.rs:510-603). Output order is (octave,
    // layer, y, x): rayon's collect keeps the sequential order.
    std::vector<OracleKeypoint> extrema(const std::vector<std::vector<ImgF>>& dog) const {
        const int border = (int)p.image_border_width;
        struct Row { size_t o, s; int y; };
        std::vector<Row> rows;
        for (size_t o = 0; o < dog.size(); ++o) {
            if (dog[o].empty()) continue;
            int H = (int)dog[o][0].h;
            for (size_t s = 1; s <= p.num_intervals; ++s) {
                if (!(s < dog[o].size() - 1)) continue;
                for (int y = border; y < H - border; ++y) rows.push_back({o, s, y});
            }
        }
        std::vector<std::vector<OracleKeypoint>> out(rows.size());
        parallel_for(rows.size(), [&](size_t r) {
            size_t o = rows[r].o, s = rows[r].s;
            int y = rows[r].y;
            const ImgF& prv = dog[o][s - 1];
            const ImgF& cur = dog[o][s];
            const ImgF& nxt = dog[o][s + 1];
            int W = (int)cur.w;
            float scale = pow2i((int)o);
            for (int x = border; x < W - border; ++x) {
                float v = pix(cur, x, y);
                bool is_max = true, is_min = true;
                for (int dz = -1; dz <= 1 && (is_max || is_min); ++dz) {
                    const ImgF& im = dz < 0 ? prv : (dz == 0 ? cur : nxt);
                    for (int dy = -1; dy <= 1 && (is_max || is_min); ++dy)
                        for (int dx = -1; dx <= 1; ++dx) {
                            if (dz == 0 && dy == 0 && dx == 0) continue;
                            float nv = pix(im, x + dx, y + dy);
                            if (v <= nv) is_max = false;
                            if (v >= nv) is_min = false;
                            if (!is_max && !is_min) break;
                        }
                }
                if (is_max || is_min) {
                    OracleKeypoint kp;
                    kp.x = ((float)x + 0.5f) * scale;
                    kp.y = ((float)y + 0.5f) * scale;
                    kp.size = 0.0f;
                    kp.angle = 0.0f;
                    kp.response = v;
                    kp.octave = (int32_t)o;
                    kp.layer = (int32_t)s;
                    out[r].push_back(kp);
                }
            }
        });
        std::vector<OracleKeypoint> all;
        for (auto& v : out) all.insert(all.end(), v.begin(), v.end());
        return all;
    }

    // solve_linear_system (src/sift.rs:478-503)
    static bool solve3(const float a[3][3], const float b[3], float x[3]) {
        float det_a = a[0][0] * (a[1][1] * a[2][2] - a[1][2] * a[2][1]) -
                      a[0][1] * (a[1][0] * a[2][2] - a[1][2] * a[2][0]) +
                      a[0][2] * (a[1][0] * a[2][1] - a[1][1] * a[2][0]);
        if (std::fabs(det_a) < 1e-10f) return false;
        float det_x = b[0] * (a[1][1] * a[2][2] - a[1][2] * a[2][1]) -
                      a[0][1] * (b[1] * a[2][2] - a[1][2] * b[2]) +
                      a[0][2] * (b[1] * a[2][1] - a[1][1] * b[2]);
        float det_y = a[0][0] * (b[1] * a[2][2] - a[1][2] * b[2]) -
                      b[0] * (a[1][0] * a[2][2] - a[1][2] * a[2][0]) +
                      a[0][2] * (a[1][0] * b[2] - b[1] * a[2][0]);
        float det_z = a[0][0] * (a[1][1] * b[2] - b[1] * a[2][1]) -
                      a[0][1] * (a[1][0] * b[2] - b[1] * a[2][0]) +
                      b[0] * (a[1][0] * a[2][1] - a[1][1] * a[2][0]);
        x[0] = det_x / det_a;
        x[1] = det_y / det_a;
        x[2] = det_z / det_a;
        return true;
    }

    // refine_and_filter_extrema (src/sift.rs:299-474): sequential, order kept.
    std::vector<OracleKeypoint> refine(const std::vector<OracleKeypoint>& cands,
                                       const std::vector<std::vector<ImgF>>& dog) const {
        std::vector<OracleKeypoint> outv;
        for (const auto& kp : cands) {
            float scale = pow2i(kp.octave);
            int cx = as_i32(kp.x / scale), cy = as_i32(kp.y / scale);
            int cl = kp.layer;
            const auto& oct = dog[(size_t)kp.octave];
            const int nl = (int)oct.size();
            for (int step = 0; step < kMaxInterpSteps; ++step) {
                if (cl < 1 || cl >= nl - 1) break;
                const ImgF& ip = oct[(size_t)cl - 1];
                const ImgF& ic = oct[(size_t)cl];
                const ImgF& in = oct[(size_t)cl + 1];
                int W = (int)ic.w, H = (int)ic.h;
                if (cx < 1 || cx >= W - 1 || cy < 1 || cy >= H - 1) break;
                float dx = (pix(ic, cx + 1, cy) - pix(ic, cx - 1, cy)) / 2.0f;
                float dy = (pix(ic, cx, cy + 1) - pix(ic, cx, cy - 1)) / 2.0f;
                float ds = (pix(in, cx, cy) - pix(ip, cx, cy)) / 2.0f;
                float c = pix(ic, cx, cy);
                float dxx = pix(ic, cx + 1, cy) + pix(ic, cx - 1, cy) - 2.0f * c;
                float dyy = pix(ic, cx, cy + 1) + pix(ic, cx, cy - 1) - 2.0f * c;
                float dss = pix(in, cx, cy) + pix(ip, cx, cy) - 2.0f * c;
                float dxy = (pix(ic, cx + 1, cy + 1) - pix(ic, cx - 1, cy + 1) - pix(ic, cx + 1, cy - 1) +
                             pix(ic, cx - 1, cy - 1)) / 4.0f;
                float dxs = (pix(in, cx + 1, cy) - pix(in, cx - 1, cy) -
                             (pix(ip, cx + 1, cy) - pix(ip, cx - 1, cy))) / 4.0f;
                float dys = (pix(in, cx, cy + 1) - pix(in, cx, cy - 1) -
                             (pix(ip, cx, cy + 1) - pix(ip, cx, cy - 1))) / 4.0f;
                const float hm[3][3] = {{dxx, dxy, dxs}, {dxy, dyy, dys}, {dxs, dys, dss}};
                const float g[3] = {-dx, -dy, -ds};
                float off[3];
                if (!solve3(hm, g, off)) break;
                if (std::fabs(off[0]) < kInterpOffsetThr && std::fabs(off[1]) < kInterpOffsetThr &&
                    std::fabs(off[2]) < kInterpOffsetThr) {
                    float val = c + 0.5f * (dx * off[0] + dy * off[1] + ds * off[2]);
                    if (std::fabs(val) < p.contrast_threshold) break;
                    float tr = dxx + dyy;
                    float trace_sq = tr * tr;
                    float det = dxx * dyy - dxy * dxy;
                    if (det <= 0.0f) break;
                    float ratio = trace_sq / det;
                    float e1 = p.edge_threshold + 1.0f;
                    float thr = (e1 * e1) / p.edge_threshold;
                    if (ratio >= thr) break;
                    float lf = (float)cl + off[2];
                    float size = p.sigma * std::pow(2.0f, (float)kp.octave + lf / (float)p.num_intervals);
                    OracleKeypoint r;
                    r.x = ((float)cx + off[0]) * scale;
                    r.y = ((float)cy + off[1]) * scale;
                    r.size = size;
                    r.angle = 0.0f;
                    r.response = val;
                    r.octave = kp.octave;
                    r.layer = as_i32(std::round(lf));
                    outv.push_back(r);
                    break;
                }
                cx = as_i32(std::round((float)cx + off[0]));
                cy = as_i32(std::round((float)cy + off[1]));
                cl = as_i32(std::round((float)cl + off[2]));
                if (cl < 0 || cl >= nl) break;
            }
        }
        return outv;
    }

    // assign_orientations (src/sift.rs:605-726): per keypoint, peaks in bin order.
    std::vector<OracleKeypoint> orientations(const std::vector<OracleKeypoint>& kps,
                                             const std::vector<std::vector<Gray>>& g) const {
        std::vector<std::vector<OracleKeypoint>> per(kps.size());
        parallel_for(kps.size(), [&](size_t i) {
            const OracleKeypoint& kp = kps[i];
            size_t o = (size_t)kp.octave;
            int li = std::max(0, std::min(kp.layer, (int)p.num_intervals + 2));
            if (o >= g.size() || (size_t)li >= g[o].size()) return;
            const Gray& im = g[o][(size_t)li];
            int W = (int)im.w, H = (int)im.h;
            float scale = pow2i(kp.octave);
            float xo = kp.x / scale, yo = kp.y / scale, so = kp.size / scale;
            if (so <= 0.0f) return;
            int radius = as_i32(std::round(kOriRadiusFactor * kOriSigmaFactor * so));
            float ws = kOriSigmaFactor * so;
            float wd = 2.0f * ws * ws;
            float hist[kOriBins] = {0};
            for (int dy = -radius; dy <= radius; ++dy)
                for (int dx = -radius; dx <= radius; ++dx) {
                    int xi = as_i32(std::round(xo + (float)dx));
                    int yi = as_i32(std::round(yo + (float)dy));
                    if (xi < 1 || xi >= W - 1 || yi < 1 || yi >= H - 1) continue;
                    float gx = gpix(im, xi + 1, yi) - gpix(im, xi - 1, yi);
                    float gy = gpix(im, xi, yi + 1) - gpix(im, xi, yi - 1);
                    float mag = std::sqrt(gx * gx + gy * gy);
                    float ang = std::atan2(gy, gx);
                    float fdx = (float)dx, fdy = (float)dy;
                    float w = std::exp(-(fdx * fdx + fdy * fdy) / wd);
                    float an = ang < 0.0f ? ang + 2.0f * kPi : ang;
                    float bf = an * (float)kOriBins / (2.0f * kPi);
                    size_t bin = (size_t)(as_usize(std::floor(bf)) % kOriBins);
                    hist[bin] += mag * w;
                }
            for (int it = 0; it < kOriSmoothIters; ++it) {
                float prev[kOriBins];
                std::memcpy(prev, hist, sizeof(hist));
                for (int b = 0; b < kOriBins; ++b) {
                    int pb = (b + kOriBins - 1) % kOriBins, nb = (b + 1) % kOriBins;
                    hist[b] = (prev[pb] + prev[b] + prev[nb]) / 3.0f;
                }
            }
            float mx = 0.0f;
            for (int b = 0; b < kOriBins; ++b) mx = std::fmax(mx, hist[b]);
            float thr = mx * kOriPeakRatio;
            for (int b = 0; b < kOriBins; ++b) {
                float cv = hist[b];
                if (!(cv >= thr)) continue;
                float pv = hist[(b + kOriBins - 1) % kOriBins], nv = hist[(b + 1) % kOriBins];
                if (cv > pv && cv > nv) {
                    float den = pv - 2.0f * cv + nv;
                    float off = std::fabs(den) > 1e-5f ? 0.5f * (pv - nv) / den : 0.0f;
                    float center = ((float)b + 0.5f) * (2.0f * kPi / (float)kOriBins);
                    float a = center + off * (2.0f * kPi / (float)kOriBins);
                    float fa = rem_euclid(a, 2.0f * kPi);
                    if (fa > kPi) fa = fa - 2.0f * kPi;
                    OracleKeypoint nk = kp;
                    nk.angle = fa;
                    per[i].push_back(nk);
                }
            }
        });
        std::vector<OracleKeypoint> all;
        for (auto& v : per) all.insert(all.end(), v.begin(), v.end());
        return all;
    }

    // get_gauss_pixel_bilinear (src/sift.rs:238-266)
    static float bilinear(const Gray& im, float x, float y) {
        float xf = std::floor(x), yf = std::floor(y);
        float xc = xf + 1.0f, yc = yf + 1.0f;
        float dx = x - xf, dy = y - yf;
        int x0 = as_i32(xf), y0 = as_i32(yf), x1 = as_i32(xc), y1 = as_i32(yc);
        float q11 = gpix(im, x0, y0), q21 = gpix(im, x1, y0);
        float q12 = gpix(im, x0, y1), q22 = gpix(im, x1, y1);
        return q11 * (1.0f - dx) * (1.0f - dy) + q21 * dx * (1.0f - dy) + q12 * (1.0f - dx) * dy +
               q22 * dx * dy;
    }

    // normalize_and_clip_descriptor (src/sift.rs:889-913)
    static void normalize_clip(float* d) {
        float s = 0.0f;
        for (int i = 0; i < kDescLen; ++i) s += d[i] * d[i];
        float norm = std::sqrt(s);
        if (norm < 1e-8f) return;
        float inv = 1.0f / norm;
        float s2 = 0.0f;
        for (int i = 0; i < kDescLen; ++i) {
            d[i] *= inv;
            d[i] = std::fmin(d[i], kDescMagThr);
            s2 += d[i] * d[i];
        }
        float n2 = std::sqrt(s2);
        if (n2 < 1e-8f) return;
        float inv2 = 1.0f / n2;
        for (int i = 0; i < kDescLen; ++i) d[i] *= inv2;
    }

    // compute (src/sift.rs:917-1060)
    void descriptor(const OracleKeypoint& kp, const std::vector<std::vector<Gray>>& g, float* hist) const {
        std::fill(hist, hist + kDescLen, 0.0f);
        size_t o = (size_t)kp.octave;
        int li = std::max(0, std::min(kp.layer, (int)p.num_intervals + 2));
        if (o >= g.size() || (size_t)li >= g[o].size()) return;
        const Gray& im = g[o][(size_t)li];
        float scale = pow2i(kp.octave);
        float xo = kp.x / scale, yo = kp.y / scale, so = kp.size / scale;
        if (so <= 0.0f) return;
        float ca = std::cos(kp.angle), sa = std::sin(kp.angle);
        float bw = kDescPatchScale * so;
        float ww = bw * (float)kDescWidth;
        float wsig = 0.5f * ww;
        float wd = 2.0f * wsig * wsig;
        int rad = as_i32(std::ceil(ww * std::sqrt(2.0f) * 0.5f));
        const float Wm1 = (float)(im.w - 1), Hm1 = (float)(im.h - 1);
        for (int dyi = -rad; dyi <= rad; ++dyi)
            for (int dxi = -rad; dxi <= rad; ++dxi) {
                float px = (float)dxi, py = (float)dyi;
                float rx = ca * px + sa * py;
                float ry = -sa * px + ca * py;
                float xb = rx / bw + (float)kDescWidth / 2.0f - 0.5f;
                float yb = ry / bw + (float)kDescWidth / 2.0f - 0.5f;
                if (!(xb > -1.0f && xb < (float)kDescWidth && yb > -1.0f && yb < (float)kDescWidth)) continue;
                float xs = xo + px, ys = yo + py;
                if (xs < 0.0f || xs >= Wm1 || ys < 0.0f || ys >= Hm1) continue;
                float gx = bilinear(im, xs + 1.0f, ys) - bilinear(im, xs - 1.0f, ys);
                float gy = bilinear(im, xs, ys + 1.0f) - bilinear(im, xs, ys - 1.0f);
                float mag = std::sqrt(gx * gx + gy * gy);
                float pa = std::atan2(gy, gx);
                float ar = rem_euclid(pa - kp.angle, 2.0f * kPi);
                float w = std::exp(-(px * px + py * py) / wd);
                float wm = mag * w;
                float ab = ar * (float)kDescBins / (2.0f * kPi);
                int xbi = as_i32(std::floor(xb)), ybi = as_i32(std::floor(yb)), abi = as_i32(std::floor(ab));
                float dxi_ = xb - (float)xbi, dyi_ = yb - (float)ybi, dai = ab - (float)abi;
                for (int i = 0; i < 2; ++i)
                    for (int j = 0; j < 2; ++j)
                        for (int k = 0; k < 2; ++k) {
                            int ix = xbi + i, iy = ybi + j;
                            int ia = ((abi + k) % kDescBins + kDescBins) % kDescBins;
                            if (ix >= 0 && ix < kDescWidth && iy >= 0 && iy < kDescWidth) {
                                float wx = i == 0 ? 1.0f - dxi_ : dxi_;
                                float wy = j == 0 ? 1.0f - dyi_ : dyi_;
                                float wa = k == 0 ? 1.0f - dai : dai;
                                float c = wm * wx * wy * wa;
                                hist[(iy * kDescWidth + ix) * kDescBins + ia] += c;
                            }
                        }
            }
        normalize_clip(hist);
    }

    // detect_and_compute_cpu steps 1-2 (src/sift.rs:1200-1214)
    Gray base_image(const Gray& gray) const {
        float amt = p.sigma > p.assumed_blur
                        ? std::sqrt(p.sigma * p.sigma - p.assumed_blur * p.assumed_blur)
                        : 0.0f;
        if (amt > 1e-4f) return gaussian_blur_f32(gray, amt);
        return gray;
    }
};

Gray make_gray(const uint8_t* img, uint32_t w, uint32_t h, uint32_t stride) {
    Gray g(w, h);
    for (uint32_t y = 0; y < h; ++y) std::memcpy(&g.px[(size_t)y * w], img + (size_t)y * stride, w);
    return g;
}

void set_threads(int threads) {
    if (threads <= 0) {
        unsigned hc = std::thread::hardware_concurrency();
        g_threads = hc ? (int)hc : 1;
    } else {
        g_threads = threads;
    }
}

void fill_result(const std::vector<OracleKeypoint>& kps, const float* desc, OracleResult* out) {
    out->n = (uint32_t)kps.size();
    out->kps = (OracleKeypoint*)std::malloc(sizeof(OracleKeypoint) * (kps.size() ? kps.size() : 1));
    if (!kps.empty()) std::memcpy(out->kps, kps.data(), sizeof(OracleKeypoint) * kps.size());
    out->desc = nullptr;
    if (desc) {
        size_t nb = sizeof(float) * kDescLen * (kps.size() ? kps.size() : 1);
        out->desc = (float*)std::malloc(nb);
        if (!kps.empty()) std::memcpy(out->desc, desc, sizeof(float) * kDescLen * kps.size());
    }
}

OracleKeypoint* copy_kps(const std::vector<OracleKeypoint>& v) {
    auto* p = (OracleKeypoint*)std::malloc(sizeof(OracleKeypoint) * (v.size() ? v.size() : 1));
    if (!v.empty()) std::memcpy(p, v.data(), sizeof(OracleKeypoint) * v.size());
    return p;
}

bool params_ok(const OracleParams* p) { return p && p->num_octaves >= 1 && p->num_intervals >= 1; }

}  // namespace

extern "C" {

void oracle_default_params(OracleParams* p) {
    oracle_new_params(p, 1.6f, 4, 3, 0.5f, 0.04f, 10.0f);
}

void oracle_new_params(OracleParams* p, float sigma, uint32_t num_octaves, uint32_t num_intervals,
                       float assumed_blur, float contrast_threshold, float edge_threshold) {
    p->sigma = sigma;
    p->num_octaves = num_octaves;
    p->num_intervals = num_intervals;
    p->assumed_blur = assumed_blur;
    p->contrast_threshold = contrast_threshold / (float)num_intervals;
    p->edge_threshold = edge_threshold;
    p->image_border_width = 5;
}

void oracle_get_blur_model(OracleBlurModel* m) { *m = g_blur_model; }
void oracle_set_blur_model(const OracleBlurModel* m) { g_blur_model = *m; }

int oracle_stages(const OracleParams* p, const uint8_t* img, uint32_t w, uint32_t h, uint32_t stride,
                  int threads, OracleStages* out) {
    if (!params_ok(p) || !out || (w && h && !img) || stride < w) return -1;
    set_threads(threads);
    Sift s{*p};
    Gray gray = make_gray(img, w, h, stride);
    Gray base = s.base_image(gray);
    auto pyr = s.gaussian_pyramid(base);
    auto dog = s.dog_pyramid(pyr);
    auto cands = s.extrema(dog);
    auto refined = s.refine(cands, dog);
    auto ori = s.orientations(refined, pyr);
    std::vector<float> desc(ori.size() * kDescLen);
    parallel_for(ori.size(), [&](size_t i) { s.descriptor(ori[i], pyr, &desc[i * kDescLen]); });

    std::memset(out, 0, sizeof(*out));
    out->num_octaves = (uint32_t)pyr.size();
    out->levels_per_octave = p->num_intervals + 3;
    out->oct_w = (uint32_t*)std::malloc(sizeof(uint32_t) * pyr.size());
    out->oct_h = (uint32_t*)std::malloc(sizeof(uint32_t) * pyr.size());
    uint64_t total = 0;
    for (size_t o = 0; o < pyr.size(); ++o) {
        out->oct_w[o] = pyr[o][0].w;
        out->oct_h[o] = pyr[o][0].h;
        total += (uint64_t)pyr[o][0].w * pyr[o][0].h * pyr[o].size();
    }
    out->pyramid_bytes = total;
    out->pyramid = (uint8_t*)std::malloc(total ? total : 1);
    uint64_t off = 0;
    for (auto& oct : pyr)
        for (auto& lv : oct) {
            if (!lv.px.empty()) std::memcpy(out->pyramid + off, lv.px.data(), lv.px.size());
            off += lv.px.size();
        }
    out->n_candidates = (uint32_t)cands.size();
    out->candidates = copy_kps(cands);
    out->n_refined = (uint32_t)refined.size();
    out->refined = copy_kps(refined);
    fill_result(ori, desc.data(), &out->result);
    return 0;
}

void oracle_stages_free(OracleStages* s) {
    if (!s) return;
    std::free(s->oct_w);
    std::free(s->oct_h);
    std::free(s->pyramid);
    std::free(s->candidates);
    std::free(s->refined);
    oracle_result_free(&s->result);
    std::memset(s, 0, sizeof(*s));
}

static int run(const OracleParams* p, const uint8_t* img, uint32_t w, uint32_t h, uint32_t stride,
               int threads, bool with_desc, OracleResult* out) {
    if (!params_ok(p) || !out || (w && h && !img) || stride < w) return -1;
    set_threads(threads);
    Sift s{*p};
    Gray gray = make_gray(img, w, h, stride);
    Gray base = s.base_image(gray);
    auto pyr = s.gaussian_pyramid(base);
    auto dog = s.dog_pyramid(pyr);
    auto cands = s.extrema(dog);
    auto refined = s.refine(cands, dog);
    auto ori = s.orientations(refined, pyr);
    if (!with_desc) {
        fill_result(ori, nullptr, out);
        return 0;
    }
    std::vector<float> desc(ori.size() * kDescLen);
    parallel_for(ori.size(), [&](size_t i) { s.descriptor(ori[i], pyr, &desc[i * kDescLen]); });
    fill_result(ori, desc.data(), out);
    return 0;
}

int oracle_detect_and_compute(const OracleParams* p, const uint8_t* img, uint32_t w, uint32_t h,
                              uint32_t stride, int threads, OracleResult* out) {
    return run(p, img, w, h, stride, threads, true, out);
}

int oracle_detect(const OracleParams* p, const uint8_t* img, uint32_t w, uint32_t h, uint32_t stride,
                  int threads, OracleResult* out) {
    return run(p, img, w, h, stride, threads, false, out);
}

void oracle_result_free(OracleResult* r) {
    if (!r) return;
    std::free(r->kps);
    std::free(r->desc);
    r->kps = nullptr;
    r->desc = nullptr;
    r->n = 0;
}

void oracle_gaussian_blur_u8(const uint8_t* in, uint32_t w, uint32_t h, float sigma, uint8_t* out) {
    Gray g = make_gray(in, w, h, w);
    Gray b = gaussian_blur_f32(g, sigma);
    if (!b.px.empty()) std::memcpy(out, b.px.data(), b.px.size());
}

int oracle_gaussian_kernel(float sigma, float* out, int cap) {
    auto k = gaussian_kernel(sigma);
    for (int i = 0; i < (int)k.size() && i < cap; ++i) out[i] = k[(size_t)i];
    return (int)k.size();
}

void oracle_resize_lanczos3_u8(const uint8_t* in, uint32_t w, uint32_t h, uint32_t nw, uint32_t nh,
                               uint8_t* out) {
    Gray g = make_gray(in, w, h, w);
    Gray r = resize_lanczos3(g, nw, nh);
    if (!r.px.empty()) std::memcpy(out, r.px.data(), r.px.size());
}

int oracle_solve3(const float* a, const float* b, float* x) {
    const float m[3][3] = {{a[0], a[1], a[2]}, {a[3], a[4], a[5]}, {a[6], a[7], a[8]}};
    return Sift::solve3(m, b, x) ? 1 : 0;
}

float oracle_bilinear(const uint8_t* img, uint32_t w, uint32_t h, float x, float y) {
    Gray g = make_gray(img, w, h, w);
    return Sift::bilinear(g, x, y);
}

int oracle_blur_sigmas(const OracleParams* p, float* out, int cap) {
    if (!params_ok(p)) return 0;
    int n = 0;
    auto put = [&](float v) {
        if (n < cap) out[n] = v;
        ++n;
    };
    float amt = p->sigma > p->assumed_blur
                    ? std::sqrt(p->sigma * p->sigma - p->assumed_blur * p->assumed_blur)
                    : 0.0f;
    put(amt > 1e-4f ? amt : 0.0f);
    float k = std::pow(2.0f, 1.0f / (float)p->num_intervals);
    std::vector<float> target;
    for (uint32_t s = 0; s < p->num_intervals + 3; ++s) target.push_back(p->sigma * powi(k, (int)s));
    for (uint32_t o = 0; o < p->num_octaves; ++o) {
        float prev = p->sigma * pow2i((int)o);
        for (uint32_t s = 1; s < p->num_intervals + 3; ++s) {
            float t = target[s] * pow2i((int)o);
            float blur = std::sqrt(t * t - prev * prev);
            put(blur < 1e-4f ? 0.0f : blur);
            prev = t;
        }
    }
    return n;
}

}  // extern "C"
