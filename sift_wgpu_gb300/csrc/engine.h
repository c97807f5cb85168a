// engine.h — the per-image SIFT engine (internal to libsiftcuda.so).
//
// One engine owns one CUDA stream and a device arena laid out per image size:
//
//   G arena    octave-major Gaussian levels, (S+3) planes per octave, each
//              plane pitch x H (pitch = width rounded up to 32 elements), f32
//              or f16 (u8-valued either way)
//   U arena    (S+3) u8 planes per octave: every level as bytes, the input
//              of the next level, of the resize and of the extrema scan
//   tmp        one u8 plane for the horizontal blur pass (largest octave)
//   ltmp       one f32 plane for the vertical Lanczos pass
//   mask       per octave S x H x ceil(W/32) ballot words of extrema
//   lists      candidates / refined / oriented keypoints and descriptors,
//              sized by capacity and grown (with a re-run) on overflow
//
// Everything stays resident across calls; the filter tables are rebuilt only
// when the image size changes. A run is a fixed sequence of launches on the
// stream with no host synchronisation until the final counters are read, so
// the same sequence is replayed from a CUDA graph per image size.
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cmath>
#include <cstring>
#include <memory>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "sift_internal.cuh"
#include "tables.h"

namespace sift {

// launchers (pyramid.cu, detect.cu, describe.cu)
template <typename TG>
int launch_blur_level(const uint8_t* in, int in_pitch, uint8_t* tmp, TG* out, uint8_t* out_u8, int pitch, int W,
                      int H, int r, const float* wts, const float* lut255, cudaStream_t st, int* launches,
                      int fused_max_radius, const ImgRef* ref = nullptr, int tile_rows = 64);
template <typename TG>
int launch_copy_level(const TG* prev, const uint8_t* prev_u8, TG* out, uint8_t* out_u8, int pitch, int W,
                      int H, cudaStream_t st);
template <typename TG>
int launch_u8_to_level(const uint8_t* img, long long stride, TG* out, uint8_t* out_u8, int pitch, int W, int H,
                       cudaStream_t st, const ImgRef* ref = nullptr);
template <typename TG>
int launch_lanczos(const uint8_t* src, int src_pitch, int W, int H, float* tmp, int tmp_pitch, TG* dst,
                   uint8_t* dst_u8, int dst_pitch, int nW, int nH, const int* vtab, const float* vw, const int* htab,
                   const float* hw, const LanczosUniform& uni, cudaStream_t st, bool fused, int* launches);
int lanczos_fused_span();
int lanczos_fused_tile();
int pixel_channels(int format);
int launch_export(const Counters* ctr, const Keypoint* kps, Counters* hctr, Keypoint* hkps, uint32_t cap,
                  cudaStream_t st);
int launch_draw_keypoints(const uint8_t* d_gray, int stride, const Keypoint* d_kps, uint32_t n, uint8_t* d_rgb,
                          int pitch, int W, int H, uint8_t r, uint8_t g, uint8_t b, cudaStream_t st);
size_t match_scratch_bytes(uint32_t nq, uint32_t nt);
const uint32_t* match_error_word(const void* scratch, uint32_t nq, uint32_t nt);
int launch_match(const float* d_q, uint32_t nq, const float* d_t, uint32_t nt, SiftCudaMatch* d_out, void* scratch,
                 cudaStream_t st);
int launch_to_luma(int format, const uint8_t* px, long long stride, int W, int H, uint8_t* out, long long out_pitch,
                   cudaStream_t st);
int launch_extrema_mask(const uint8_t* u8arena, const float* lut255, const EntryTable& tab, const OctaveDev& od,
                        int e, int border, uint32_t* words, cudaStream_t st);
int extrema_tiles(int W, int H);
int launch_extrema_mask_flat(const uint8_t* u8arena, const float* lut255, const EntryTable& tab, int e0, int n_e,
                             const uint32_t* tile_pref, uint32_t n_tiles, int border, uint32_t* words,
                             cudaStream_t st);
int launch_dog_dense(const uint8_t* u8arena, const float* lut255, const PyramidDev& pyr, int o, int l, float* out,
                     cudaStream_t st);
int launch_emit(const uint8_t* u8arena, const float* lut255, const EntryTable& tab, int e0, int n_e,
                long long n_words, const uint32_t* words, const uint32_t* cand_off, Keypoint* cands, uint32_t cap,
                Counters* ctr, cudaStream_t st);
int launch_refine(const uint8_t* u8arena, const float* lut255, const EntryTable& tab, float sigma, float contrast,
                  float edge, const Keypoint* cands, Keypoint* refined_at, uint32_t* keep, uint32_t cap,
                  OctCounters* oc, cudaStream_t st);
template <typename TG>
int launch_orientation(const TG* arena, const EntryTable& tab, const float* lut255, const Keypoint* refined_at,
                       const uint32_t* keep, uint32_t ncap, OctCounters* oc, float* ori_angle, uint32_t* ori_count,
                       int grid, int persist_ctas, cudaStream_t st);
int launch_orient_emit(const Keypoint* refined_at, uint32_t ncap, int o, Counters* ctr, const float* ori_angle,
                       const uint32_t* ori_count, const uint32_t* ori_off, Keypoint* oriented, uint32_t cap,
                       cudaStream_t st);
template <typename TG>
int launch_descriptor(const TG* arena, const EntryTable& tab, const Keypoint* oriented,
                      OctCounters* oc, float* desc, uint32_t cap, float* hdesc, uint32_t hcap, int grid,
                      int persist_ctas, cudaStream_t st);
// Error reporting (engine.cu): the calling thread's sift_cuda_last_error.
extern thread_local std::string g_last_error;
int fail(int code, const std::string& msg);
int cuda_fail(cudaError_t e, const char* what);
int report_error(int code, const char* msg);

#define CK(call, what)                              \
    do {                                            \
        cudaError_t e_ = (call);                    \
        if (e_ != cudaSuccess) return cuda_fail(e_, what); \
    } while (0)

struct DevMem {
    void* p = nullptr;
    size_t bytes = 0;
    ~DevMem() { release(); }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
    }
    cudaError_t ensure(size_t n) {
        if (n <= bytes && p) return cudaSuccess;
        release();
        if (n == 0) n = 16;
        cudaError_t e = cudaMalloc(&p, n);
        if (e == cudaSuccess) bytes = n;
        return e;
    }
    template <typename T>
    T* as() const {
        return (T*)p;
    }
};

struct HostPinned {
    void* p = nullptr;
    size_t bytes = 0;
    ~HostPinned() { release(); }
    void release() {
        if (p) cudaFreeHost(p);
        p = nullptr;
        bytes = 0;
    }
    cudaError_t ensure(size_t n) {
        if (n <= bytes && p) return cudaSuccess;
        release();
        if (n == 0) n = 16;
        cudaError_t e = cudaHostAlloc(&p, n, cudaHostAllocDefault);
        if (e == cudaSuccess) bytes = n;
        return e;
    }
    template <typename T>
    T* as() const {
        return (T*)p;
    }
};

inline size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

struct LevelBlur {
    float sigma;   // 0 = copy
    int radius;
    size_t woff;   // offset in the weight table
};

struct Engine {
    SiftCudaParams p{};
    SiftCudaOptions opt{};
    cudaStream_t st = nullptr;

    // geometry of the current arena
    uint32_t W = 0, H = 0;
    bool have_geom = false;
    PyramidDev pyr{};
    long long n_words = 0;
    size_t g_elems = 0, u_bytes = 0, tmp_bytes = 0, ltmp_elems = 0;
    size_t lut_off = 0;  // v / 255 table (256 floats) in d_wts
    LevelBlur base{};
    std::vector<std::vector<LevelBlur>> lv;  // [o][s-1]
    struct LTab {
        size_t vtab, vw, htab, hw;  // element offsets in d_ltab / d_lw
        bool fused;                 // every output tile's source window fits the fused kernel
        LanczosUniform uni;         // the interior of a 2x resize (empty otherwise)
    };
    // Outputs [*lo, *hi) of a resize axis whose taps start at 2 o - 5, number
    // kLz2xTaps and equal the middle output's bit for bit (a 2x resize away
    // from the borders); w receives those taps. Empty unless src = 2 dst.
    static void uniform_2x(const AxisTaps& t, uint32_t src, int* lo, int* hi, float* w) {
        *lo = *hi = 0;
        const int n = (int)t.left.size();
        if (n < 8 || src != 2u * (uint32_t)n) return;
        const int m = n / 2;
        auto same = [&](int o) {
            if (t.count[o] != kLz2xTaps || t.left[o] != 2 * o - 5) return false;
            return std::memcmp(&t.w[t.woff[o]], &t.w[t.woff[m]], sizeof(float) * kLz2xTaps) == 0;
        };
        if (!same(m)) return;
        int a = m, b = m + 1;
        while (a > 0 && same(a - 1)) --a;
        while (b < n && same(b)) ++b;
        *lo = a;
        *hi = b;
        std::memcpy(w, &t.w[t.woff[m]], sizeof(float) * kLz2xTaps);
    }
    std::vector<LTab> ltab;  // [o] for o -> o+1

    // Lists. Octave o owns [cb[o], cb[o] + cap_c[o]) of the candidate-sized
    // lists (candidates, refined, keep flags, orientation scratch) and its own
    // scan scratch; the output lists (oriented keypoints, descriptors) are
    // shared, octave after octave.
    std::vector<uint32_t> cap_c, cb;
    std::vector<size_t> pb, tb;  // scan-state (64-bit words) and horizontal-pass buffer offsets
    size_t scan_words = 0;       // scan state of the run, zeroed at its start
    uint32_t cap_cand = 0, cap_ori = 0;

    DevMem d_px;  // colour input before its luma conversion
    DevMem d_mq, d_mt, d_mo, d_ms;  // descriptor matching: query, train, result, scratch
    DevMem d_dg, d_dk, d_drgb;       // drawing: grey input, keypoints, RGB output
    DevMem d_img, d_G, d_U, d_tmp, d_tmpo, d_ltmp, d_wts, d_ltab, d_lw;
    DevMem d_words, d_cand_off, d_keep, d_scan;
    DevMem d_ents;  // the entry table: pyr.oct[0 .. num_octaves) in device memory
    EntryTable tab() const { return EntryTable{d_ents.as<OctaveDev>(), pyr.num_octaves, pyr.S}; }
    DevMem d_cands, d_refined_at, d_ori_angle, d_ori_count, d_ori_off, d_oriented, d_desc, d_ctr;
    HostPinned h_ctr, h_kps, h_desc;
    // Host calls: the run ends with an export kernel that writes counters,
    // keypoints and descriptors into this mapped buffer (layout: Counters |
    // keypoints[cap_x] | descriptors[cap_x]), sized from the last count.
    HostPinned hx;
    uint32_t cap_x = 0, last_n = 0;
    // descriptors [0, desc_on_host) of the last run live only in the export
    // buffer (a host call writes them there from the descriptor stage)
    uint32_t desc_on_host = 0;
    Counters* hx_dctr = nullptr;  // device addresses of the three parts
    Keypoint* hx_dkps = nullptr;
    float* hx_ddesc = nullptr;
    Counters* hx_ctr() const { return hx.as<Counters>(); }
    Keypoint* hx_kps() const { return (Keypoint*)(hx.as<char>() + align_up(sizeof(Counters), 256)); }
    float* hx_desc() const {
        return (float*)(hx.as<char>() + align_up(sizeof(Counters), 256) + align_up((size_t)cap_x * sizeof(Keypoint), 256));
    }
    size_t img_pitch = 0;
    // The image cell the base level reads (ImgRef): set by every upload.
    // Pageable caller images are read where they are when the device reads
    // pageable host memory coherently (a GB300's Grace host), saving the
    // staged copy; pinned and device images are copied to d_img (a DMA copy
    // is faster than the base level's staging reads over the host link).
    DevMem d_ref;
    HostPinned h_ref;
    int pageable_reads = -1;  // device attribute, read once
    bool image_in_place = false, ref_valid = false;
    uint32_t launches = 0;
    bool last_desc = true;

    // Launch-shape knobs (set by the batch autotuner; the defaults are the
    // tuned values for single 1080p..4096 images): the largest blur radius
    // that runs as one fused kernel, the persistent grids of the
    // orientation and descriptor kernels in CTAs per SM, and the height of
    // the fused level kernel's tiles (64 or 32 rows).
    struct Tuning {
        int fused_max_radius = 8;
        int ori_ctas_per_sm = 4;
        int desc_ctas_per_sm = 8;
        int level_tile_rows = 64;
        bool operator==(const Tuning& o) const {
            return fused_max_radius == o.fused_max_radius && ori_ctas_per_sm == o.ori_ctas_per_sm &&
                   desc_ctas_per_sm == o.desc_ctas_per_sm && level_tile_rows == o.level_tile_rows;
        }
    } tune{};

    // One stream per octave for the level DAG and its events (see enqueue_t),
    // and the CUDA graph the whole run is replayed from.
    std::vector<cudaStream_t> st_oct;
    std::vector<cudaEvent_t> ev_level, ev_ori, ev_done;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t gexec = nullptr;
    struct GraphKey {
        uint32_t W = 0, H = 0, cap_ori = 0, cap_x = 0;  // cap_x 0: no export node
        std::vector<uint32_t> cap_c;
        bool with_desc = false;
        Tuning tune{};
        bool operator==(const GraphKey& o) const {
            return W == o.W && H == o.H && cap_ori == o.cap_ori && cap_c == o.cap_c && with_desc == o.with_desc &&
                   tune == o.tune && cap_x == o.cap_x;
        }
    } gkey{};
    uint32_t graph_launches = 0;

    void drop_graph() {
        if (gexec) cudaGraphExecDestroy(gexec);
        if (graph) cudaGraphDestroy(graph);
        gexec = nullptr;
        graph = nullptr;
    }

    // Per-stage device time accounting (sift_cuda_profile_*): events recorded
    // on the stream at the stage boundaries of every run while enabled.
    static constexpr int kStages = 4;
    bool prof = false;
    std::vector<cudaEvent_t> ev_free;
    std::vector<std::vector<cudaEvent_t>> ev_runs;  // kStages + 1 events per run

    ~Engine() {
        drop_graph();
        for (auto& r : ev_runs)
            for (auto e : r) cudaEventDestroy(e);
        for (auto e : ev_free) cudaEventDestroy(e);
        for (auto* v : {&ev_level, &ev_ori, &ev_done})
            for (auto e : *v)
                if (e) cudaEventDestroy(e);
        for (auto q : st_oct)
            if (q) cudaStreamDestroy(q);
        if (st) cudaStreamDestroy(st);
    }

    cudaEvent_t take_event() {
        if (!ev_free.empty()) {
            cudaEvent_t e = ev_free.back();
            ev_free.pop_back();
            return e;
        }
        cudaEvent_t e = nullptr;
        cudaEventCreate(&e);
        return e;
    }
    void mark(std::vector<cudaEvent_t>* run) {
        if (!prof) return;
        cudaEvent_t e = take_event();
        if (e) {
            cudaEventRecord(e, st);
            run->push_back(e);
        }
    }
    int profile_read(float* ms, uint32_t n, uint32_t* runs) {
        CK(cudaStreamSynchronize(st), "synchronize");
        std::vector<double> acc(kStages, 0.0);
        uint32_t nr = 0;
        for (auto& r : ev_runs) {
            if ((int)r.size() == kStages + 1) {
                for (int k = 0; k < kStages; ++k) {
                    float t = 0.0f;
                    cudaEventElapsedTime(&t, r[k], r[k + 1]);
                    acc[k] += t;
                }
                ++nr;
            }
            for (auto e : r) ev_free.push_back(e);
        }
        ev_runs.clear();
        for (uint32_t k = 0; k < n && k < (uint32_t)kStages; ++k) ms[k] = (float)acc[k];
        if (runs) *runs = nr;
        return 0;
    }

    // CUDA stream priority of the engine (0 = default; lower is more
    // urgent): octave 0's stream runs at it, the other streams one step more
    // urgent (see init).
    int priority = 0;

    bool f16() const { return opt.storage == SIFT_CUDA_STORAGE_F16; }
    bool u8() const { return opt.storage == SIFT_CUDA_STORAGE_U8; }

    // Device bytes held by the engine's arenas and lists.
    size_t device_bytes() const {
        size_t t = 0;
        for (const DevMem* m : {&d_img, &d_G, &d_U, &d_tmp, &d_tmpo, &d_ltmp, &d_wts, &d_ltab, &d_lw, &d_words,
                                &d_cand_off, &d_keep, &d_scan, &d_cands, &d_refined_at,
                                &d_ori_angle, &d_ori_count, &d_ori_off, &d_oriented, &d_desc, &d_ctr})
            t += m->bytes;
        return t;
    }
    // bytes of a stored level value; u8 storage stores nothing beyond the u8 planes
    size_t g_elem_size() const { return u8() ? 0 : (f16() ? 2 : 4); }

    int set_device() {
        CK(cudaSetDevice(opt.device), "cudaSetDevice");
        return 0;
    }

    int init() {
        if (int rc = set_device()) return rc;
        // Octave 0's stream runs at the engine's priority, the pyramid's main
        // stream and the smaller octaves' streams one step more urgent: while
        // octave 0's orientation and descriptors fill the device, the other
        // octaves' levels and short latency-bound chains are scheduled first
        // instead of being left as a tail after them.
        int least = 0, greatest = 0;
        CK(cudaDeviceGetStreamPriorityRange(&least, &greatest), "stream priority range");
        const int base = std::min(std::max(priority, greatest), least);
        const int urgent = std::max(base - 1, greatest);
        CK(cudaStreamCreateWithPriority(&st, cudaStreamNonBlocking, urgent), "cudaStreamCreate");
        st_oct.assign(kMaxOctaves, nullptr);
        for (size_t o = 0; o < st_oct.size(); ++o)
            CK(cudaStreamCreateWithPriority(&st_oct[o], cudaStreamNonBlocking, o == 0 ? base : urgent),
               "cudaStreamCreate");
        for (auto* v : {&ev_level, &ev_ori, &ev_done}) {
            v->assign(kMaxOctaves, nullptr);
            for (auto& e : *v) CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "cudaEventCreate");
        }
        CK(h_ctr.ensure(sizeof(Counters)), "cudaHostAlloc(counters)");
        CK(d_ctr.ensure(sizeof(Counters)), "cudaMalloc(counters)");
        return 0;
    }

    long long octave_words(int o) const { return (long long)pyr.S * pyr.oct[o].H * pyr.oct[o].nw; }

    // Lays out the arena for a width x height image and builds the tables.
    int ensure_geometry(uint32_t w, uint32_t h) {
        if (have_geom && w == W && h == H) return 0;
        const int O = (int)p.num_octaves, S = (int)p.num_intervals;
        if (O > kMaxOctaves) return fail(SIFT_CUDA_ERR_UNSUPPORTED, "num_octaves above 16 is not supported");
        PyramidDev g{};
        g.num_octaves = O;
        g.S = S;
        g.levels = S + 3;
        size_t goff = 0, uoff = 0, wbase = 0, tmpb = 0, lt = 0, tmpo = 0;
        std::vector<size_t> tbo(O, 0);
        uint32_t ow = w, oh = h;
        for (int o = 0; o < O; ++o) {
            OctaveDev& od = g.oct[o];
            od.W = (int)ow;
            od.H = (int)oh;
            od.pitch = (int)align_up(std::max<uint32_t>(ow, 1), 32);
            od.nw = (int)((ow + 31) / 32);
            od.plane = (long long)od.pitch * oh;
            od.g_off = (long long)goff;
            od.word_base = (long long)wbase;
            od.u_off = (long long)uoff;
            od.octave = o;
            od.image = 0;
            goff += (size_t)od.plane * (S + 3);
            uoff += (size_t)od.plane * (S + 3);
            wbase += (size_t)S * oh * od.nw;
            tmpb = std::max(tmpb, (size_t)od.pitch * oh);
            tbo[o] = tmpo;
            tmpo += align_up((size_t)od.pitch * oh, 256);
            if (o + 1 < O) lt = std::max(lt, (size_t)od.pitch * (oh / 2));
            ow /= 2;
            oh /= 2;
        }
        // blur tables
        BlurPlan bp = blur_plan(p);
        std::vector<float> wts;
        auto add_blur = [&](float sigma) {
            LevelBlur b{sigma, 0, wts.size()};
            if (sigma > 0.0f) {
                auto k = gaussian_kernel(sigma);
                b.radius = (int)(k.size() / 2);
                wts.insert(wts.end(), k.begin(), k.end());
                while (wts.size() % 4) wts.push_back(0.0f);
            }
            return b;
        };
        base = add_blur(bp.base);
        lv.assign(O, {});
        for (int o = 0; o < O; ++o)
            for (int s = 1; s < S + 3; ++s) lv[o].push_back(add_blur(bp.level[o][s - 1]));
        // v / 255 in f32 (IEEE division): the normalised level value and the
        // DoG operands (src/sift.rs:92-124)
        const size_t lutw = wts.size();
        for (int v = 0; v < 256; ++v) wts.push_back((float)v / 255.0f);
        // Lanczos tables
        std::vector<int> itab;
        std::vector<float> ftab;
        ltab.assign(O, LTab{0, 0, 0, 0, false, LanczosUniform{}});
        auto max_span = [](const AxisTaps& t) {
            const int T = lanczos_fused_tile(), n = (int)t.left.size();
            int m = 0;
            for (int a = 0; a < n; a += T) {
                const int b = std::min(a + T, n) - 1;
                m = std::max(m, t.left[b] + t.count[b] - t.left[a]);
            }
            return m;
        };
        for (int o = 0; o + 1 < O; ++o) {
            const OctaveDev& a = g.oct[o];
            const int nW = g.oct[o + 1].W, nH = g.oct[o + 1].H;
            if (a.W == 0 || a.H == 0 || nW == 0 || nH == 0) continue;
            AxisTaps tv = lanczos_axis((uint32_t)a.H, (uint32_t)nH);
            AxisTaps th = lanczos_axis((uint32_t)a.W, (uint32_t)nW);
            LTab t;
            t.vtab = itab.size();
            itab.insert(itab.end(), tv.left.begin(), tv.left.end());
            itab.insert(itab.end(), tv.count.begin(), tv.count.end());
            itab.insert(itab.end(), tv.woff.begin(), tv.woff.end());
            t.vw = ftab.size();
            ftab.insert(ftab.end(), tv.w.begin(), tv.w.end());
            t.htab = itab.size();
            itab.insert(itab.end(), th.left.begin(), th.left.end());
            itab.insert(itab.end(), th.count.begin(), th.count.end());
            itab.insert(itab.end(), th.woff.begin(), th.woff.end());
            t.hw = ftab.size();
            ftab.insert(ftab.end(), th.w.begin(), th.w.end());
            t.fused = max_span(tv) <= lanczos_fused_span() && max_span(th) <= lanczos_fused_span();
            t.uni = LanczosUniform{};
            uniform_2x(th, (uint32_t)a.W, &t.uni.x0, &t.uni.x1, t.uni.wh);
            uniform_2x(tv, (uint32_t)a.H, &t.uni.y0, &t.uni.y1, t.uni.wv);
            if (t.uni.x0 >= t.uni.x1 || t.uni.y0 >= t.uni.y1) t.uni.x0 = t.uni.x1 = t.uni.y0 = t.uni.y1 = 0;
            ltab[o] = t;
        }
        // allocate
        drop_graph();
        n_words = (long long)wbase;
        CK(d_G.ensure(goff * g_elem_size()), "cudaMalloc(G)");
        CK(d_U.ensure(uoff + 64), "cudaMalloc(u8 levels)");
        CK(d_tmp.ensure(std::max<size_t>(tmpb, 16)), "cudaMalloc(tmp)");
        CK(d_tmpo.ensure(std::max<size_t>(tmpo, 16)), "cudaMalloc(tmp per octave)");
        CK(d_ltmp.ensure(std::max<size_t>(lt, 4) * sizeof(float)), "cudaMalloc(ltmp)");
        CK(d_wts.ensure(std::max<size_t>(wts.size(), 4) * sizeof(float)), "cudaMalloc(wts)");
        CK(d_ltab.ensure(std::max<size_t>(itab.size(), 4) * sizeof(int)), "cudaMalloc(ltab)");
        CK(d_lw.ensure(std::max<size_t>(ftab.size(), 4) * sizeof(float)), "cudaMalloc(lw)");
        const size_t nwb = std::max<size_t>((size_t)n_words, 1) * sizeof(uint32_t);
        CK(d_words.ensure(nwb), "cudaMalloc(words)");
        CK(d_ents.ensure(sizeof(OctaveDev) * (size_t)std::max(O, 1)), "cudaMalloc(entries)");
        if (O > 0)
            CK(cudaMemcpyAsync(d_ents.p, g.oct, sizeof(OctaveDev) * (size_t)O, cudaMemcpyHostToDevice, st),
               "H2D entries");
        CK(d_cand_off.ensure(nwb), "cudaMalloc(cand_off)");
        if (!wts.empty())
            CK(cudaMemcpyAsync(d_wts.p, wts.data(), wts.size() * sizeof(float), cudaMemcpyHostToDevice, st), "H2D wts");
        if (!itab.empty())
            CK(cudaMemcpyAsync(d_ltab.p, itab.data(), itab.size() * sizeof(int), cudaMemcpyHostToDevice, st),
               "H2D ltab");
        if (!ftab.empty())
            CK(cudaMemcpyAsync(d_lw.p, ftab.data(), ftab.size() * sizeof(float), cudaMemcpyHostToDevice, st), "H2D lw");
        CK(cudaStreamSynchronize(st), "table upload");
        pyr = g;
        g_elems = goff;
        u_bytes = uoff;
        lut_off = lutw;
        tmp_bytes = tmpb;
        ltmp_elems = lt;
        tb = tbo;
        W = w;
        H = h;
        have_geom = true;
        // Initial list capacities: 1/64 of each octave's scanned positions
        // (measured densities on natural and synthetic images are far below
        // it), at least 1024; grown on overflow.
        cap_c.assign(O, 0);
        for (int o = 0; o < O; ++o)
            cap_c[o] = (uint32_t)std::min<size_t>(std::max<size_t>((size_t)octave_words(o) * 32 / 64, 1024), 1u << 28);
        size_t tot = 0;
        for (auto c : cap_c) tot += c;
        cap_ori = std::max<uint32_t>(cap_ori, (uint32_t)std::min<size_t>(tot, 1u << 30));
        return ensure_lists();
    }

    int ensure_lists() {
        drop_graph();
        const int O = pyr.num_octaves;
        cb.assign(O, 0);
        pb.assign(O, 0);
        size_t c = 0, pp = 0;
        for (int o = 0; o < O; ++o) {
            cb[o] = (uint32_t)c;
            c += cap_c[o];
            // two scans per octave: the candidate words, then the orientation counts
            pb[o] = pp;
            pp += scan_state_words((size_t)octave_words(o)) + scan_state_words((size_t)cap_c[o]);
        }
        scan_words = pp;
        if (c > (1u << 30)) return fail(SIFT_CUDA_ERR_CAPACITY, "keypoint lists above 2^30");
        cap_cand = (uint32_t)c;
        const size_t kp = sizeof(Keypoint);
        CK(d_cands.ensure((size_t)cap_cand * kp), "cudaMalloc(cands)");
        CK(d_refined_at.ensure((size_t)cap_cand * kp), "cudaMalloc(refined_at)");
        CK(d_ori_angle.ensure((size_t)cap_cand * kOriMaxPeaks * sizeof(float)), "cudaMalloc(ori_angle)");
        CK(d_ori_count.ensure((size_t)cap_cand * sizeof(uint32_t)), "cudaMalloc(ori_count)");
        CK(d_ori_off.ensure((size_t)cap_cand * sizeof(uint32_t)), "cudaMalloc(ori_off)");
        CK(d_keep.ensure((size_t)cap_cand * sizeof(uint32_t)), "cudaMalloc(keep)");
        CK(d_oriented.ensure((size_t)cap_ori * kp), "cudaMalloc(oriented)");
        CK(d_desc.ensure((size_t)cap_ori * kDescLen * sizeof(float)), "cudaMalloc(desc)");
        CK(d_scan.ensure(std::max<size_t>(pp, 1) * sizeof(unsigned long long)), "cudaMalloc(scan state)");
        return 0;
    }

    // The run as a DAG (dag) or in stage order on one stream (profiling):
    //   st        counters, base level, octave o levels 1..S, Lanczos(o) ->
    //             octave o+1 ...
    //   st_oct[o] after level S of octave o: levels S+1..S+2, the extrema
    //             mask, the ordered candidate list, refinement, orientation;
    //             then, once octaves 0..o-1 know their oriented counts, the
    //             output slots and the descriptors of octave o.
    //   st        waits for every octave's chain.
    // Octave 0's descriptors (most of the work) overlap the smaller octaves'
    // pyramid. Levels on st_oct[o] use their own horizontal-pass buffer.
    template <typename TG>
    int enqueue_t(const uint8_t* img, long long stride, bool with_desc, bool dag, bool exp) {
        const int O = pyr.num_octaves, S = pyr.S;
        TG* G = u8() ? (TG*)d_U.p : d_G.as<TG>();  // u8 storage: the levels are the u8 planes
        const float* wts = d_wts.as<float>();
        const float* lut = wts + lut_off;
        uint8_t* U = d_U.as<uint8_t>();
        Counters* ctr = d_ctr.as<Counters>();
        launches = 0;
        auto ok = [&](int rc) {
            ++launches;
            return rc;
        };
        std::vector<cudaEvent_t> run_ev;
        mark(&run_ev);
        CK(cudaMemsetAsync(d_ctr.p, 0, sizeof(Counters), st), "memset counters");
        CK(cudaMemsetAsync(d_scan.p, 0, scan_words * sizeof(unsigned long long), st), "memset scan state");
        int O_used = 0;
        for (int o = 0; o < O && pyr.oct[o].W > 0 && pyr.oct[o].H > 0; ++o) O_used = o + 1;

        auto level = [&](int o, int s, cudaStream_t q, uint8_t* tmp) -> int {
            const OctaveDev& od = pyr.oct[o];
            const LevelBlur& b = lv[o][s - 1];
            const TG* prev = G + od.g_off + (long long)(s - 1) * od.plane;
            TG* out = G + od.g_off + (long long)s * od.plane;
            const uint8_t* prev_u8 = U + od.u_off + (long long)(s - 1) * od.plane;
            uint8_t* out_u8 = U + od.u_off + (long long)s * od.plane;
            if (b.sigma <= 0.0f) {
                if (ok(launch_copy_level<TG>(prev, prev_u8, out, out_u8, od.pitch, od.W, od.H, q)))
                    return cuda_fail(cudaGetLastError(), "copy level");
                return 0;
            }
            int nl = 0;
            if (launch_blur_level<TG>(prev_u8, od.pitch, tmp, out, out_u8, od.pitch, od.W, od.H, b.radius,
                                      wts + b.woff, lut, q, &nl, tune.fused_max_radius, nullptr,
                                      tune.level_tile_rows))
                return cuda_fail(cudaGetLastError(), "blur level");
            launches += nl;
            return 0;
        };
        auto lanczos = [&](int o) -> int {
            const OctaveDev& od = pyr.oct[o];
            const OctaveDev& nx = pyr.oct[o + 1];
            const LTab& t = ltab[o];
            const int* it = d_ltab.as<int>();
            const float* ft = d_lw.as<float>();
            int nl = 0;
            if (launch_lanczos<TG>(U + od.u_off + (long long)S * od.plane, od.pitch, od.W, od.H, d_ltmp.as<float>(),
                                   od.pitch, G + nx.g_off, U + nx.u_off, nx.pitch, nx.W, nx.H, it + t.vtab, ft + t.vw,
                                   it + t.htab, ft + t.hw, t.uni, st, t.fused, &nl))
                return cuda_fail(cudaGetLastError(), "lanczos");
            launches += nl;
            return 0;
        };
        // (b)+(c): extrema, ordered candidates, refinement of octave o
        auto detect = [&](int o, cudaStream_t q) -> int {
            const OctaveDev& od = pyr.oct[o];
            OctCounters* oc = &ctr->oct[o];
            unsigned long long* sstate = d_scan.as<unsigned long long>() + pb[o];
            const long long nwo = octave_words(o);
            if (od.nw > 0 && ok(launch_extrema_mask(U, lut, tab(), od, o, (int)p.image_border_width,
                                                    d_words.as<uint32_t>(), q)))
                return cuda_fail(cudaGetLastError(), "extrema mask");
            if (scan_exclusive(d_words.as<uint32_t>() + od.word_base, SCAN_POPC,
                               d_cand_off.as<uint32_t>() + od.word_base, (size_t)nwo, nullptr, &oc->n_cand, sstate,
                               &ctr->overflow, q))
                return cuda_fail(cudaGetLastError(), "scan candidates");
            launches += nwo > 0 ? 1 : 0;
            if (ok(launch_emit(U, lut, tab(), o, 1, nwo, d_words.as<uint32_t>() + od.word_base,
                               d_cand_off.as<uint32_t>() + od.word_base, d_cands.as<Keypoint>() + cb[o], cap_c[o], ctr,
                               q)))
                return cuda_fail(cudaGetLastError(), "emit");
            if (ok(launch_refine(U, lut, tab(), p.sigma, p.contrast_threshold, p.edge_threshold,
                                 d_cands.as<Keypoint>() + cb[o], d_refined_at.as<Keypoint>() + cb[o],
                                 d_keep.as<uint32_t>() + cb[o], cap_c[o], oc, q)))
                return cuda_fail(cudaGetLastError(), "refine");
            return 0;
        };
        // (d) orientation histograms of the kept candidate slots and their scan
        auto orient = [&](int o, cudaStream_t q) -> int {
            OctCounters* oc = &ctr->oct[o];
            // one warp-item per 8 candidate slots, 4 per warp; the last
            // 152 x ori_ctas_per_sm CTAs drain whatever is left
            const int grid = (int)std::max<uint32_t>(cap_c[o] / 64, 32);
            if (ok(launch_orientation<TG>(G, tab(), lut, d_refined_at.as<Keypoint>() + cb[o], d_keep.as<uint32_t>() + cb[o],
                                          cap_c[o], oc, d_ori_angle.as<float>() + (size_t)cb[o] * kOriMaxPeaks,
                                          d_ori_count.as<uint32_t>() + cb[o], grid, 152 * tune.ori_ctas_per_sm, q)))
                return cuda_fail(cudaGetLastError(), "orientation");
            unsigned long long* sstate =
                d_scan.as<unsigned long long>() + pb[o] + scan_state_words((size_t)octave_words(o));
            if (scan_exclusive(d_ori_count.as<uint32_t>() + cb[o], SCAN_U32, d_ori_off.as<uint32_t>() + cb[o],
                               (size_t)cap_c[o], &oc->n_cand, &oc->n_ori, sstate, &ctr->overflow, q))
                return cuda_fail(cudaGetLastError(), "scan orientations");
            launches += 1;
            return 0;
        };
        // output slots of octave o (after octaves 0..o-1) and its descriptors
        auto emit_out = [&](int o, cudaStream_t q) -> int {
            if (ok(launch_orient_emit(d_refined_at.as<Keypoint>() + cb[o], cap_c[o], o, ctr,
                                      d_ori_angle.as<float>() + (size_t)cb[o] * kOriMaxPeaks,
                                      d_ori_count.as<uint32_t>() + cb[o], d_ori_off.as<uint32_t>() + cb[o],
                                      d_oriented.as<Keypoint>(), cap_ori, q)))
                return cuda_fail(cudaGetLastError(), "orientation emit");
            return 0;
        };
        auto describe = [&](int o, cudaStream_t q) -> int {
            if (!with_desc) return 0;
            // two keypoints per CTA for 1/8 of the candidate capacity; the
            // last 152 x desc_ctas_per_sm CTAs drain whatever is left
            const int grid = (int)std::max<uint32_t>(cap_c[o] / 16, 64);
            // host calls: descriptors below cap_x go straight into the mapped
            // export buffer while the stage runs, the rest to d_desc
            if (ok(launch_descriptor<TG>(G, tab(), d_oriented.as<Keypoint>(), &ctr->oct[o], d_desc.as<float>(), cap_ori,
                                         exp ? hx_ddesc : nullptr, exp ? cap_x : 0u, grid,
                                         152 * tune.desc_ctas_per_sm, q)))
                return cuda_fail(cudaGetLastError(), "descriptor");
            return 0;
        };

        const OctaveDev& o0 = pyr.oct[0];
        if (O_used > 0) {
            // base image (src/sift.rs:1204-1214)
            if (base.sigma > 0.0f) {
                int nl = 0;
                if (launch_blur_level<TG>(img, (int)stride, d_tmp.as<uint8_t>(), G + o0.g_off, U + o0.u_off,
                                          o0.pitch, o0.W, o0.H, base.radius, wts + base.woff, lut, st,
                                          &nl, tune.fused_max_radius, d_ref.as<ImgRef>(), tune.level_tile_rows))
                    return cuda_fail(cudaGetLastError(), "blur (base)");
                launches += nl;
            } else {
                if (ok(launch_u8_to_level<TG>(img, stride, G + o0.g_off, U + o0.u_off, o0.pitch, o0.W, o0.H, st,
                                              d_ref.as<ImgRef>())))
                    return cuda_fail(cudaGetLastError(), "base copy");
            }
        }
        if (dag) {
            for (int o = 0; o < O_used; ++o) {
                cudaStream_t q = st_oct[o];
                uint8_t* tmp_o = d_tmpo.as<uint8_t>() + tb[o];
                for (int s = 1; s <= S; ++s)
                    if (int rc = level(o, s, st, d_tmp.as<uint8_t>())) return rc;
                CK(cudaEventRecord(ev_level[o], st), "event record");
                CK(cudaStreamWaitEvent(q, ev_level[o], 0), "stream wait");
                for (int s = S + 1; s < S + 3; ++s)
                    if (int rc = level(o, s, q, tmp_o)) return rc;
                if (int rc = detect(o, q)) return rc;
                if (int rc = orient(o, q)) return rc;
                CK(cudaEventRecord(ev_ori[o], q), "event record");
                for (int k = 0; k < o; ++k) CK(cudaStreamWaitEvent(q, ev_ori[k], 0), "stream wait");
                if (int rc = emit_out(o, q)) return rc;
                if (int rc = describe(o, q)) return rc;
                CK(cudaEventRecord(ev_done[o], q), "event record");
                if (o + 1 < O_used)
                    if (int rc = lanczos(o)) return rc;
            }
            for (int o = 0; o < O_used; ++o) CK(cudaStreamWaitEvent(st, ev_done[o], 0), "stream wait");
        } else {
            // Stage by stage. Inside the pyramid stage, as in the graph, the
            // levels above S of octave o (which the next octave does not
            // need) run on the octave's stream beside the next octave's
            // chain; the stage ends when every level exists.
            for (int o = 0; o < O_used; ++o) {
                for (int s = 1; s <= S; ++s)
                    if (int rc = level(o, s, st, d_tmp.as<uint8_t>())) return rc;
                CK(cudaEventRecord(ev_level[o], st), "event record");
                CK(cudaStreamWaitEvent(st_oct[o], ev_level[o], 0), "stream wait");
                for (int s = S + 1; s < S + 3; ++s)
                    if (int rc = level(o, s, st_oct[o], d_tmpo.as<uint8_t>() + tb[o])) return rc;
                CK(cudaEventRecord(ev_done[o], st_oct[o]), "event record");
                if (o + 1 < O_used)
                    if (int rc = lanczos(o)) return rc;
            }
            for (int o = 0; o < O_used; ++o) CK(cudaStreamWaitEvent(st, ev_done[o], 0), "stream wait");
            mark(&run_ev);
            for (int o = 0; o < O_used; ++o)
                if (int rc = detect(o, st)) return rc;
            mark(&run_ev);
            for (int o = 0; o < O_used; ++o)
                if (int rc = orient(o, st)) return rc;
            for (int o = 0; o < O_used; ++o)
                if (int rc = emit_out(o, st)) return rc;
            mark(&run_ev);
            for (int o = 0; o < O_used; ++o)
                if (int rc = describe(o, st)) return rc;
        }
        if (O_used == 0) {
            mark(&run_ev);
            mark(&run_ev);
            mark(&run_ev);
        }
        mark(&run_ev);
        if (prof) ev_runs.push_back(std::move(run_ev));
        if (exp) {
            // counters and keypoints; the descriptors are there already
            if (ok(launch_export(ctr, d_oriented.as<Keypoint>(), hx_dctr, hx_dkps, cap_x, st)))
                return cuda_fail(cudaGetLastError(), "export");
        }
        last_desc = with_desc;
        return 0;
    }

    int enqueue(const uint8_t* img, long long stride, bool with_desc, bool dag, bool exp) {
        if (u8()) return enqueue_t<uint8_t>(img, stride, with_desc, dag, exp);
        return f16() ? enqueue_t<__half>(img, stride, with_desc, dag, exp)
                     : enqueue_t<float>(img, stride, with_desc, dag, exp);
    }

    // Mapped export buffer for at least n keypoints (host calls). It grows
    // with twice the headroom so that images of one size with more keypoints
    // than the last seldom force a reallocation (and a graph re-capture).
    int ensure_export(uint32_t n) {
        if (hx.p && n <= cap_x) return 0;
        const uint32_t cap = std::max<uint32_t>(2 * n + 4096, 2 * cap_x);
        hx.release();
        void* ptr = nullptr;
        const size_t bytes = align_up(sizeof(Counters), 256) + align_up((size_t)cap * sizeof(Keypoint), 256) +
                             (size_t)cap * kDescLen * sizeof(float);
        CK(cudaHostAlloc(&ptr, bytes, cudaHostAllocMapped), "cudaHostAlloc(export)");
        hx.p = ptr;
        hx.bytes = bytes;
        cap_x = cap;
        CK(cudaHostGetDevicePointer((void**)&hx_dctr, hx_ctr(), 0), "cudaHostGetDevicePointer");
        CK(cudaHostGetDevicePointer((void**)&hx_dkps, hx_kps(), 0), "cudaHostGetDevicePointer");
        CK(cudaHostGetDevicePointer((void**)&hx_ddesc, hx_desc(), 0), "cudaHostGetDevicePointer");
        return 0;
    }

    // After a run that ended with the export (its counters c read from the
    // buffer): a run with more keypoints than the buffer holds grows it and
    // moves its results there — keypoints from d_oriented, descriptors below
    // the old capacity from the old buffer, the rest from d_desc. Records
    // what the buffer holds.
    int settle_export(const Counters& c, bool with_desc) {
        const uint32_t n = c.n_oriented;
        if (n > cap_x) {
            const uint32_t head = cap_x;
            std::vector<float> d_head;
            if (with_desc) d_head.assign(hx_desc(), hx_desc() + (size_t)head * kDescLen);
            if (int rc = ensure_export(n)) return rc;
            *hx_ctr() = c;
            CK(cudaMemcpy(hx_kps(), d_oriented.p, sizeof(Keypoint) * n, cudaMemcpyDeviceToHost), "D2H kps");
            if (with_desc) {
                std::memcpy(hx_desc(), d_head.data(), sizeof(float) * d_head.size());
                CK(cudaMemcpy(hx_desc() + (size_t)head * kDescLen, d_desc.as<float>() + (size_t)head * kDescLen,
                              sizeof(float) * kDescLen * (n - head), cudaMemcpyDeviceToHost),
                   "D2H desc");
            }
        }
        last_n = n;
        desc_on_host = with_desc ? n : 0;
        return 0;
    }

    // One run on the image in d_img: replayed from the CUDA graph of this
    // size (captured on first use), or launched in order with stage events
    // when profiling.
    // exp: end the run with the export into the mapped buffer (host calls).
    int run(bool with_desc, bool exp = false) {
        const long long stride = (long long)img_pitch;
        desc_on_host = 0;
        if (prof) return enqueue(d_img.as<uint8_t>(), stride, with_desc, false, exp);
        GraphKey key;
        key.W = W;
        key.H = H;
        key.cap_ori = cap_ori;
        key.cap_c = cap_c;
        key.with_desc = with_desc;
        key.tune = tune;
        key.cap_x = exp ? cap_x : 0;
        if (!gexec || !(key == gkey)) {
            drop_graph();
            CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal), "begin capture");
            int rc = enqueue(d_img.as<uint8_t>(), stride, with_desc, true, exp);
            cudaGraph_t g = nullptr;
            cudaError_t e = cudaStreamEndCapture(st, &g);
            if (rc) {
                if (g) cudaGraphDestroy(g);
                return rc;
            }
            if (e != cudaSuccess) return cuda_fail(e, "end capture");
            graph = g;
            // each kernel node keeps the priority of the stream it was captured on
            CK(cudaGraphInstantiate(&gexec, graph, cudaGraphInstantiateFlagUseNodePriority), "graph instantiate");
            gkey = key;
            graph_launches = launches;
        }
        launches = graph_launches;
        CK(cudaGraphLaunch(gexec, st), "graph launch");
        return 0;
    }

    // Grows the lists that the counters c of a finished run overflowed;
    // *retry tells that the run must be repeated.
    int grow_from(const Counters& c, bool* retry) {
        *retry = false;
        if (c.overflow & 8u) return fail(SIFT_CUDA_ERR_CUDA, "a prefix-scan wait ran out (the run was abandoned)");
        bool grow = false;
        for (int o = 0; o < pyr.num_octaves; ++o) {
            const uint32_t n = c.oct[o].n_cand;
            if (n > cap_c[o]) {
                const size_t nc = (size_t)n + n / 4 + 1024;
                if (nc > (1u << 28)) return fail(SIFT_CUDA_ERR_CAPACITY, "candidate list above 2^28");
                cap_c[o] = (uint32_t)nc;
                grow = true;
            }
        }
        if ((c.overflow & 4u) || c.n_oriented > cap_ori) {
            const size_t no = std::max<size_t>((size_t)cap_ori * 2, (size_t)c.n_oriented + c.n_oriented / 4 + 1024);
            if (no > (1u << 30)) return fail(SIFT_CUDA_ERR_CAPACITY, "keypoint list above 2^30");
            cap_ori = (uint32_t)no;
            grow = true;
        }
        if (grow) {
            if (int rc = ensure_lists()) return rc;
            *retry = true;
        }
        return 0;
    }

    int upload(const uint8_t* img, uint32_t w, uint32_t h, uint32_t stride, cudaMemcpyKind kind) {
        const size_t pitch = align_up(std::max<uint32_t>(w, 1), 128);
        if (pitch != img_pitch || !d_img.p || d_img.bytes < pitch * std::max<uint32_t>(h, 1)) drop_graph();
        img_pitch = pitch;
        CK(d_img.ensure(img_pitch * std::max<uint32_t>(h, 1)), "cudaMalloc(image)");
        if (!d_ref.p) {
            CK(d_ref.ensure(sizeof(ImgRef)), "cudaMalloc(image cell)");
            CK(h_ref.ensure(sizeof(ImgRef)), "cudaHostAlloc(image cell)");
        }
        if (pageable_reads < 0) {
            int v = 0;
            if (cudaDeviceGetAttribute(&v, cudaDevAttrPageableMemoryAccess, opt.device) != cudaSuccess) v = 0;
            pageable_reads = v == 1 ? 1 : 0;
        }
        // in place: a pageable host image starting and striding on 16 bytes
        // (the level kernel's staging loads), a blurred base level
        bool in_place = false;
        if (pageable_reads && kind == cudaMemcpyHostToDevice && img && w && h && base.sigma > 0.0f &&
            ((uintptr_t)img & 15) == 0 && (stride & 15) == 0 && stride <= (1u << 30)) {
            cudaPointerAttributes a{};
            if (cudaPointerGetAttributes(&a, img) == cudaSuccess) in_place = a.type == cudaMemoryTypeUnregistered;
            else cudaGetLastError();
        }
        image_in_place = in_place;
        const ImgRef cell = in_place ? ImgRef{img, (long long)stride} : ImgRef{d_img.as<uint8_t>(), (long long)img_pitch};
        if (!in_place && w && h && img)
            CK(cudaMemcpy2DAsync(d_img.p, img_pitch, img, stride, w, h, kind, st), "copy image");
        // The cell is rewritten only when it changes: a run that reads it is
        // ordered after the copy on the stream, and a changed cell comes from
        // a host call, which has waited for the previous run to end.
        ImgRef* r = h_ref.as<ImgRef>();
        if (!ref_valid || r->ptr != cell.ptr || r->pitch != cell.pitch) {
            *r = cell;
            CK(cudaMemcpyAsync(d_ref.p, h_ref.p, sizeof(ImgRef), cudaMemcpyHostToDevice, st), "H2D image cell");
            ref_valid = true;
        }
        return 0;
    }

    int detect_host(const uint8_t* img, uint32_t w, uint32_t h, uint32_t stride, bool with_desc,
                    SiftCudaResult* out, bool view = false, int format = SIFT_CUDA_PIXELS_GRAY8) {
        if (int rc = set_device()) return rc;
        if (int rc = ensure_geometry(w, h)) return rc;
        if (format == SIFT_CUDA_PIXELS_GRAY8) {
            if (int rc = upload(img, w, h, stride, cudaMemcpyHostToDevice)) return rc;
        } else {
            // colour bytes to the device, luma into the image plane
            const size_t ch = (size_t)pixel_channels(format), row = (size_t)w * ch;
            const size_t pitch = align_up(std::max<size_t>(row, 1), 128);
            CK(d_px.ensure(pitch * std::max<uint32_t>(h, 1)), "cudaMalloc(colour image)");
            if (int rc = upload(nullptr, w, h, 0, cudaMemcpyHostToDevice)) return rc;
            if (w && h) {
                CK(cudaMemcpy2DAsync(d_px.p, pitch, img, stride, row, h, cudaMemcpyHostToDevice, st), "copy pixels");
                if (launch_to_luma(format, d_px.as<uint8_t>(), (long long)pitch, (int)w, (int)h, d_img.as<uint8_t>(),
                                   (long long)img_pitch, st))
                    return cuda_fail(cudaGetLastError(), "luma conversion");
            }
        }
        if (int rc = ensure_export(last_n ? last_n : 4096)) return rc;
        for (int attempt = 0; attempt < 8; ++attempt) {
            if (int rc = run(with_desc, true)) return rc;
            CK(cudaStreamSynchronize(st), "run");
            const Counters c = *hx_ctr();
            *h_ctr.as<Counters>() = c;
            bool retry = false;
            if (int rc = grow_from(c, &retry)) return rc;
            if (retry) continue;
            if (int rc = settle_export(c, with_desc)) return rc;
            return view ? fetch_view(with_desc, out) : fetch(with_desc, out);
        }
        return fail(SIFT_CUDA_ERR_CAPACITY, "keypoint lists kept overflowing");
    }

    // Results of a host call, already in the mapped export buffer; out points
    // at them (valid until the next call).
    int fetch_view(bool with_desc, SiftCudaResult* out) {
        out->n = h_ctr.as<Counters>()->n_oriented;
        out->kps = (SiftCudaKeypoint*)hx_kps();
        out->desc = with_desc ? hx_desc() : nullptr;
        return 0;
    }

    int fetch(bool with_desc, SiftCudaResult* out) {
        const uint32_t n = h_ctr.as<Counters>()->n_oriented;
        out->n = n;
        out->kps = (SiftCudaKeypoint*)std::malloc(sizeof(SiftCudaKeypoint) * std::max<uint32_t>(n, 1));
        out->desc = with_desc ? (float*)std::malloc(sizeof(float) * kDescLen * std::max<uint32_t>(n, 1)) : nullptr;
        if (!out->kps || (with_desc && !out->desc)) {
            std::free(out->kps);
            std::free(out->desc);
            out->kps = nullptr;
            out->desc = nullptr;
            out->n = 0;
            return fail(SIFT_CUDA_ERR_OUT_OF_MEMORY, "host allocation of the result");
        }
        if (n == 0) return 0;
        copy_out(out->kps, hx_kps(), sizeof(Keypoint) * n);
        if (with_desc) copy_out(out->desc, hx_desc(), sizeof(float) * kDescLen * n);
        return 0;
    }

    // A result copy of several MB over a few host threads: one thread moves
    // a fraction of the host's memory bandwidth.
    static void copy_out(void* dst, const void* src, size_t bytes) {
        constexpr size_t kChunk = 2u << 20;
        const size_t hw = std::max<size_t>(std::thread::hardware_concurrency(), 1);
        const size_t nt = std::min<size_t>(std::min<size_t>(4, bytes / kChunk), hw);
        if (nt <= 1) {
            std::memcpy(dst, src, bytes);
            return;
        }
        const size_t per = ((bytes + nt - 1) / nt + 4095) & ~(size_t)4095;
        std::vector<std::thread> th;
        for (size_t i = 1; i < nt && i * per < bytes; ++i) {
            const size_t a = i * per, b = std::min(bytes, a + per);
            th.emplace_back([=] { std::memcpy((char*)dst + a, (const char*)src + a, b - a); });
        }
        std::memcpy(dst, src, std::min(per, bytes));
        for (auto& t : th) t.join();
    }
};

}  // namespace sift
