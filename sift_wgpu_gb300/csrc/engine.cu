// engine.cu — error state and the C ABI of the per-image engine (engine.h).
#include "engine.h"

namespace sift {

thread_local std::string g_last_error;

int fail(int code, const std::string& msg) {
    g_last_error = msg;
    return code;
}

int cuda_fail(cudaError_t e, const char* what) {
    std::string m = std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")";
    return fail(e == cudaErrorMemoryAllocation ? SIFT_CUDA_ERR_OUT_OF_MEMORY
                                               : (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver
                                                      ? SIFT_CUDA_ERR_NO_DEVICE
                                                      : SIFT_CUDA_ERR_CUDA),
                m);
}

// Sets the calling thread's sift_cuda_last_error message from another
// translation unit of the library; returns code.
int report_error(int code, const char* msg) { return fail(code, msg ? std::string(msg) : std::string()); }


}  // namespace sift

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
using sift::Engine;

struct SiftCudaEngine {
    Engine e;
};

namespace {
bool params_valid(const SiftCudaParams* p, std::string* why) {
    if (!p) {
        *why = "params is NULL";
        return false;
    }
    if (p->num_octaves < 1 || p->num_octaves > (uint32_t)sift::kMaxOctaves) {
        *why = "num_octaves must be in [1, 16]";
        return false;
    }
    if (p->num_intervals < 1 || p->num_intervals > 16) {
        *why = "num_intervals must be in [1, 16]";
        return false;
    }
    if (!(p->sigma > 0.0f) || !(p->assumed_blur >= 0.0f) || !(p->edge_threshold > 0.0f) ||
        !(p->contrast_threshold >= 0.0f)) {
        *why = "sigma and edge_threshold must be positive, assumed_blur and contrast_threshold non-negative";
        return false;
    }
    return true;
}
}  // namespace

extern "C" {

void sift_cuda_params_new(SiftCudaParams* out, float sigma, uint32_t num_octaves, uint32_t num_intervals,
                          float assumed_blur, float contrast_threshold, float edge_threshold) {
    if (!out) return;
    out->sigma = sigma;
    out->num_octaves = num_octaves;
    out->num_intervals = num_intervals;
    out->assumed_blur = assumed_blur;
    out->contrast_threshold = contrast_threshold / (float)num_intervals;
    out->edge_threshold = edge_threshold;
    out->image_border_width = 5;
}

void sift_cuda_params_default(SiftCudaParams* out) { sift_cuda_params_new(out, 1.6f, 4, 3, 0.5f, 0.04f, 10.0f); }

void sift_cuda_options_default(SiftCudaOptions* out) {
    if (!out) return;
    std::memset(out, 0, sizeof(*out));
    out->device = 0;
    out->storage = SIFT_CUDA_STORAGE_U8;
}

const char* sift_cuda_last_error(void) { return sift::g_last_error.c_str(); }

int sift_cuda_create(const SiftCudaParams* params, const SiftCudaOptions* opts, SiftCudaEngine** out) {
    sift::g_last_error.clear();
    if (!out) return sift::fail(SIFT_CUDA_ERR_INVALID_ARGUMENT, "out is NULL");
    *out = nullptr;
    std::string why;
    if (!params_valid(params, &why)) return sift::fail(SIFT_CUDA_ERR_INVALID_ARGUMENT, why);
    SiftCudaOptions o;
    sift_cuda_options_default(&o);
    if (opts) o = *opts;
    if (o.storage != SIFT_CUDA_STORAGE_F32 && o.storage != SIFT_CUDA_STORAGE_F16 && o.storage != SIFT_CUDA_STORAGE_U8)
        return sift::fail(SIFT_CUDA_ERR_INVALID_ARGUMENT, "unknown storage mode");
    if (o.level_tile_rows != 0 && o.level_tile_rows != 32 && o.level_tile_rows != 64)
        return sift::fail(SIFT_CUDA_ERR_INVALID_ARGUMENT, "level_tile_rows must be 0, 32 or 64");
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0)
        return sift::fail(SIFT_CUDA_ERR_NO_DEVICE, std::string("no CUDA device: ") + cudaGetErrorString(e));
    if (o.device < 0 || o.device >= ndev) return sift::fail(SIFT_CUDA_ERR_INVALID_ARGUMENT, "device ordinal out of range");
    auto* eng = new (std::nothrow) SiftCudaEngine();
    if (!eng) return sift::fail(SIFT_CUDA_ERR_OUT_OF_MEMORY, "engine allocation");
    eng->e.p = *params;
    eng->e.opt = o;
    if (o.level_tile_rows) eng->e.tune.level_tile_rows = o.level_tile_rows;
    if (int rc = eng->e.init()) {
        delete eng;
        return rc;
    }
    *out = eng;
    return 0;
}

void sift_cuda_destroy(SiftCudaEngine* engine) {
    if (!engine) return;
    cudaSetDevice(engine->e.opt.device);
    if (engine->e.st) cudaStreamSynchronize(engine->e.st);
    delete engine;
}

static int check_image(SiftCudaEngine* engine, const uint8_t* img, uint32_t w, uint32_t h, uint32_t stride,
                       SiftCudaResult* out) {
    if (out) {
        out->n = 0;
        out->kps = nullptr;
        out->desc = nullptr;
    }
    if (!engine) return sift::fail(SIFT_CUDA_ERR_INVALID_ARGUMENT, "engine is NULL");
    if ((w && h && !img) || stride < w)
        return sift::fail(SIFT_CUDA_ERR_INVALID_ARGUMENT, "image pointer is NULL or stride < width");
    if (w > 65535u || h > 65535u) return sift::fail(SIFT_CUDA_ERR_UNSUPPORTED, "image sides above 65535");
    return 0;
}

int sift_cuda_detect_and_compute(SiftCudaEngine* engine, const uint8_t* img, uint32_t width, uint32_t height,
                                 uint32_t stride, SiftCudaResult* out) {
    sift::g_last_error.clear();
    if (!out) return sift::fail(SIFT_CUDA_ERR_INVALID_ARGUMENT, "out is NULL");
    if (int rc = check_image(engine, img, width, height, stride, out)) return rc;
    return engine->e.detect_host(img, width, height, stride, true, out);
}

int sift_cuda_detect_and_compute_view(SiftCudaEngine* engine, const uint8_t* img, uint32_t width, uint32_t height,
                                      uint32_t stride, SiftCudaResult* out) {
    sift::g_last_error.clear();
    if (!out) return sift::fail(SIFT_CUDA_ERR_INVALID_ARGUMENT, "out is NULL");
    if (int rc = check_image(engine, img, width, height, stride, out)) return rc;
    return engine->e.detect_host(img, width, height, stride, true, out, true);
}

int sift_cuda_detect(SiftCudaEngine* engine, const uint8_t* img, uint32_t width, uint32_t height, uint32_t stride,
                     SiftCudaResult* out) {
    sift::g_last_error.clear();
    if (!out) return sift::fail(SIFT_CUDA_ERR_INVALID_ARGUMENT, "out is NULL");
    if (int rc = check_image(engine, img, width, height, stride, out)) return rc;
    return engine->e.detect_host(img, width, height, stride, false, out);
}

int sift_cuda_detect_and_compute_pixels(SiftCudaEngine* engine, const uint8_t* pixels, uint32_t width,
                                        uint32_t height, uint32_t stride, int32_t format, SiftCudaResult* out) {
    sift::g_last_error.clear();
    if (!out) return sift::fail(SIFT_CUDA_ERR_INVALID_ARGUMENT, "out is NULL");
    const int ch = sift::pixel_channels(format);
    if (ch == 0) return sift::fail(SIFT_CUDA_ERR_INVALID_ARGUMENT, "unknown pixel format");
    if ((uint64_t)stride < (uint64_t)width * (uint64_t)ch)
        return sift::fail(SIFT_CUDA_ERR_INVALID_ARGUMENT, "stride < width x channels");
    if (int rc = check_image(engine, pixels, width, height, stride, out)) return rc;
    return engine->e.detect_host(pixels, width, height, stride, true, out, false, format);
}

int sift_cuda_to_luma(const uint8_t* d_pixels, uint32_t width, uint32_t height, uint32_t stride, int32_t format,
                      uint8_t* d_out, uint32_t out_stride, void* stream) {
    sift::g_last_error.clear();
    const int ch = sift::pixel_channels(format);
    if (ch <= 1) return sift::fail(SIFT_CUDA_ERR_INVALID_ARGUMENT, "format must be a colour format");
    if (width == 0 || height == 0) return 0;
    if (!d_pixels || !d_out || (uint64_t)stride < (uint64_t)width * ch || out_stride < width)
        return sift::fail(SIFT_CUDA_ERR_INVALID_ARGUMENT, "NULL pointer or stride too small");
    if (sift::launch_to_luma(format, d_pixels, stride, (int)width, (int)height, d_out, out_stride,
                             (cudaStream_t)stream))
        return sift::cuda_fail(cudaGetLastError(), "luma conversion");
    return 0;
}

void sift_cuda_result_free(SiftCudaResult* r) {
    if (!r) return;
    std::free(r->kps);
    std::free(r->desc);
    r->kps = nullptr;
    r->desc = nullptr;
    r->n = 0;
}

int sift_cuda_run_device(SiftCudaEngine* engine, const uint8_t* d_img, uint32_t width, uint32_t height,
                         uint32_t stride, int with_descriptors) {
    sift::g_last_error.clear();
    if (int rc = check_image(engine, d_img, width, height, stride, nullptr)) return rc;
    Engine& e = engine->e;
    if (int rc = e.set_device()) return rc;
    if (int rc = e.ensure_geometry(width, height)) return rc;
    if (int rc = e.upload(d_img, width, height, stride, cudaMemcpyDeviceToDevice)) return rc;
    return e.run(with_descriptors != 0);
}

int sift_cuda_device_outputs(SiftCudaEngine* engine, const uint32_t** d_count, const SiftCudaKeypoint** d_kps,
                             const float** d_desc) {
    if (!engine) return sift::fail(SIFT_CUDA_ERR_INVALID_ARGUMENT, "engine is NULL");
    Engine& e = engine->e;
    if (d_count) *d_count = e.d_ctr.p ? &e.d_ctr.as<sift::Counters>()->n_oriented : nullptr;
    if (d_kps) *d_kps = e.d_oriented.as<SiftCudaKeypoint>();
    if (d_desc) *d_desc = e.d_desc.as<float>();
    return 0;
}

size_t sift_cuda_match_scratch_bytes(uint32_t n_query, uint32_t n_train) {
    return sift::match_scratch_bytes(n_query, n_train);
}

int sift_cuda_match_device(const float* d_query, uint32_t n_query, const float* d_train, uint32_t n_train,
                           SiftCudaMatch* d_out, void* d_scratch, void* stream) {
    sift::g_last_error.clear();
    if (n_query == 0) return 0;
    if (!d_query || !d_out || !d_scratch || (n_train && !d_train))
        return sift::fail(SIFT_CUDA_ERR_INVALID_ARGUMENT, "a matching buffer is NULL");
    if (((uintptr_t)d_query | (uintptr_t)d_train) & 15)
        return sift::fail(SIFT_CUDA_ERR_INVALID_ARGUMENT, "descriptor arrays must be 16-byte aligned");
    if (sift::launch_match(d_query, n_query, d_train, n_train, d_out, d_scratch, (cudaStream_t)stream))
        return sift::cuda_fail(cudaGetLastError(), "match");
    return 0;
}

int sift_cuda_match(SiftCudaEngine* engine, const float* query, uint32_t n_query, const float* train,
                    uint32_t n_train, SiftCudaMatch* out) {
    sift::g_last_error.clear();
    if (!engine) return sift::fail(SIFT_CUDA_ERR_INVALID_ARGUMENT, "engine is NULL");
    if (n_query == 0) return 0;
    if (!query || !out || (n_train && !train)) return sift::fail(SIFT_CUDA_ERR_INVALID_ARGUMENT, "a matching buffer is NULL");
    Engine& e = engine->e;
    if (int rc = e.set_device()) return rc;
    const size_t qb = (size_t)n_query * sift::kDescLen * sizeof(float), tb = (size_t)n_train * sift::kDescLen * sizeof(float);
    if (e.d_mq.ensure(qb) != cudaSuccess || e.d_mt.ensure(std::max<size_t>(tb, 16)) != cudaSuccess ||
        e.d_mo.ensure((size_t)n_query * sizeof(SiftCudaMatch)) != cudaSuccess ||
        e.d_ms.ensure(sift::match_scratch_bytes(n_query, n_train)) != cudaSuccess)
        return sift::cuda_fail(cudaGetLastError(), "cudaMalloc(match)");
    cudaStream_t st = e.st;
    if (cudaMemcpyAsync(e.d_mq.p, query, qb, cudaMemcpyHostToDevice, st) != cudaSuccess ||
        (tb && cudaMemcpyAsync(e.d_mt.p, train, tb, cudaMemcpyHostToDevice, st) != cudaSuccess))
        return sift::cuda_fail(cudaGetLastError(), "H2D descriptors");
    if (sift::launch_match(e.d_mq.as<float>(), n_query, e.d_mt.as<float>(), n_train, e.d_mo.as<SiftCudaMatch>(),
                           e.d_ms.p, st))
        return sift::cuda_fail(cudaGetLastError(), "match");
    uint32_t err = 0;
    if (cudaMemcpyAsync(out, e.d_mo.p, (size_t)n_query * sizeof(SiftCudaMatch), cudaMemcpyDeviceToHost, st) !=
            cudaSuccess ||
        cudaMemcpyAsync(&err, sift::match_error_word(e.d_ms.p, n_query, n_train), sizeof(err), cudaMemcpyDeviceToHost,
                        st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return sift::cuda_fail(cudaGetLastError(), "match results");
    if (err) return sift::fail(SIFT_CUDA_ERR_CUDA, "matching: a tensor-core pipeline wait ran out (no results)");
    return 0;
}

int sift_cuda_draw_keypoints(SiftCudaEngine* engine, const uint8_t* gray, uint32_t width, uint32_t height,
                             uint32_t stride, const SiftCudaKeypoint* kps, uint32_t n, uint8_t r, uint8_t g,
                             uint8_t b, uint8_t* rgb_out, uint32_t out_stride) {
    sift::g_last_error.clear();
    if (!engine) return sift::fail(SIFT_CUDA_ERR_INVALID_ARGUMENT, "engine is NULL");
    if (width == 0 || height == 0) return 0;
    if (!gray || !rgb_out || (n && !kps)) return sift::fail(SIFT_CUDA_ERR_INVALID_ARGUMENT, "a drawing buffer is NULL");
    if (stride < width || out_stride < 3ull * width || width > (1u << 30) / 3)
        return sift::fail(SIFT_CUDA_ERR_INVALID_ARGUMENT, "stride below the row size");
    Engine& e = engine->e;
    if (int rc = e.set_device()) return rc;
    const size_t pitch = ((size_t)width * 3 + 127) & ~(size_t)127;
    if (e.d_dg.ensure((size_t)width * height) != cudaSuccess || e.d_drgb.ensure(pitch * height) != cudaSuccess ||
        e.d_dk.ensure(std::max<size_t>((size_t)n * sizeof(SiftCudaKeypoint), 16)) != cudaSuccess)
        return sift::cuda_fail(cudaGetLastError(), "cudaMalloc(draw)");
    cudaStream_t st = e.st;
    if (cudaMemcpy2DAsync(e.d_dg.p, width, gray, stride, width, height, cudaMemcpyHostToDevice, st) != cudaSuccess ||
        (n && cudaMemcpyAsync(e.d_dk.p, kps, (size_t)n * sizeof(SiftCudaKeypoint), cudaMemcpyHostToDevice, st) !=
                  cudaSuccess))
        return sift::cuda_fail(cudaGetLastError(), "H2D draw");
    if (sift::launch_draw_keypoints(e.d_dg.as<uint8_t>(), (int)width, e.d_dk.as<sift::Keypoint>(), n,
                                    e.d_drgb.as<uint8_t>(), (int)pitch, (int)width, (int)height, r, g, b, st))
        return sift::cuda_fail(cudaGetLastError(), "draw");
    if (cudaMemcpy2DAsync(rgb_out, out_stride, e.d_drgb.p, pitch, (size_t)width * 3, height, cudaMemcpyDeviceToHost,
                          st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return sift::cuda_fail(cudaGetLastError(), "D2H draw");
    return 0;
}

int sift_cuda_synchronize(SiftCudaEngine* engine) {
    if (!engine) return sift::fail(SIFT_CUDA_ERR_INVALID_ARGUMENT, "engine is NULL");
    cudaError_t e = cudaStreamSynchronize(engine->e.st);
    if (e != cudaSuccess) return sift::cuda_fail(e, "synchronize");
    return 0;
}

void* sift_cuda_stream(SiftCudaEngine* engine) { return engine ? (void*)engine->e.st : nullptr; }

uint32_t sift_cuda_last_launch_count(SiftCudaEngine* engine) { return engine ? engine->e.launches : 0; }

uint32_t sift_cuda_last_image_in_place(SiftCudaEngine* engine) {
    return engine && engine->e.image_in_place ? 1u : 0u;
}

int sift_cuda_profile_enable(SiftCudaEngine* engine, int enable) {
    if (!engine) return sift::fail(SIFT_CUDA_ERR_INVALID_ARGUMENT, "engine is NULL");
    engine->e.prof = enable != 0;
    return 0;
}

int sift_cuda_profile_read(SiftCudaEngine* engine, float* stage_ms, uint32_t n_stages, uint32_t* runs) {
    if (!engine || (!stage_ms && n_stages)) return sift::fail(SIFT_CUDA_ERR_INVALID_ARGUMENT, "bad arguments");
    return engine->e.profile_read(stage_ms, n_stages, runs);
}

int sift_cuda_debug_stage(SiftCudaEngine* engine, int stage, void* out, uint64_t capacity, uint64_t* count) {
    if (!engine || !count) return sift::fail(SIFT_CUDA_ERR_INVALID_ARGUMENT, "engine or count is NULL");
    Engine& e = engine->e;
    if (!e.have_geom) return sift::fail(SIFT_CUDA_ERR_INVALID_ARGUMENT, "no run yet");
    if (cudaStreamSynchronize(e.st) != cudaSuccess) return sift::cuda_fail(cudaGetLastError(), "synchronize");
    sift::Counters c;
    if (cudaMemcpy(&c, e.d_ctr.p, sizeof(c), cudaMemcpyDeviceToHost) != cudaSuccess)
        return sift::cuda_fail(cudaGetLastError(), "D2H counters");
    const sift::PyramidDev& g = e.pyr;
    if (stage == SIFT_CUDA_STAGE_DOG) {
        // No DoG plane is stored: the detection forms DoG(l) =
        // G_{l+1}/255 - G_l/255 (src/sift.rs:92-124) from the u8 level planes
        // where it reads it. This read-back runs the device function the
        // candidate emission and the refinement use (DogFromU8) over every
        // pixel of every layer.
        const int L = g.S + 2;
        uint64_t total = 0;
        for (int o = 0; o < g.num_octaves; ++o) total += (uint64_t)g.oct[o].W * g.oct[o].H * L;
        *count = total;
        if (!out) return 0;
        size_t most = 0;
        for (int o = 0; o < g.num_octaves; ++o) most = std::max(most, (size_t)g.oct[o].W * g.oct[o].H);
        sift::DevMem tmp;
        if (tmp.ensure(std::max<size_t>(most, 1) * sizeof(float)) != cudaSuccess)
            return sift::cuda_fail(cudaGetLastError(), "cudaMalloc(DoG read-back)");
        const float* lut = e.d_wts.as<float>() + e.lut_off;
        uint64_t pos = 0;
        for (int o = 0; o < g.num_octaves && pos < capacity; ++o) {
            const sift::OctaveDev& od = g.oct[o];
            if (od.W == 0 || od.H == 0) continue;
            const uint64_t npx = (uint64_t)od.W * od.H;
            for (int l = 0; l < L && pos < capacity; ++l) {
                if (sift::launch_dog_dense(e.d_U.as<uint8_t>(), lut, g, o, l, tmp.as<float>(), e.st))
                    return sift::cuda_fail(cudaGetLastError(), "DoG read-back");
                const uint64_t n = std::min<uint64_t>(npx, capacity - pos);
                if (cudaMemcpyAsync((float*)out + pos, tmp.p, n * sizeof(float), cudaMemcpyDeviceToHost, e.st) !=
                        cudaSuccess ||
                    cudaStreamSynchronize(e.st) != cudaSuccess)
                    return sift::cuda_fail(cudaGetLastError(), "D2H stage");
                pos += n;
            }
        }
        return 0;
    }
    if (stage == SIFT_CUDA_STAGE_PYRAMID) {
        const int L = g.S + 3;
        uint64_t total = 0;
        for (int o = 0; o < g.num_octaves; ++o) total += (uint64_t)g.oct[o].W * g.oct[o].H * L;
        *count = total;
        if (!out) return 0;
        uint64_t pos = 0;
        std::vector<unsigned char> buf;
        for (int o = 0; o < g.num_octaves; ++o) {
            const sift::OctaveDev& od = g.oct[o];
            if (od.W == 0 || od.H == 0) continue;
            for (int l = 0; l < L; ++l) {
                // the stored levels (the u8 planes themselves in u8 storage)
                const size_t es = e.u8() ? 1 : e.g_elem_size();
                const char* src = e.u8() ? (const char*)e.d_U.p + (size_t)(od.u_off + (long long)l * od.plane)
                                         : (const char*)e.d_G.p + (size_t)(od.g_off + (long long)l * od.plane) * es;
                buf.resize((size_t)od.W * od.H * es);
                if (cudaMemcpy2D(buf.data(), (size_t)od.W * es, src, (size_t)od.pitch * es, (size_t)od.W * es, od.H,
                                 cudaMemcpyDeviceToHost) != cudaSuccess)
                    return sift::cuda_fail(cudaGetLastError(), "D2H stage");
                const size_t npx = (size_t)od.W * od.H;
                for (size_t q = 0; q < npx && pos < capacity; ++q, ++pos) {
                    if (es == 1) {
                        ((uint8_t*)out)[pos] = buf[q];
                    } else if (es == 4) {
                        ((uint8_t*)out)[pos] = (uint8_t)std::lrint(((const float*)buf.data())[q] * 255.0f);
                    } else {
                        ((uint8_t*)out)[pos] = (uint8_t)__half2float(((const __half*)buf.data())[q]);
                    }
                }
            }
        }
        return 0;
    }
    const sift::Keypoint* src = nullptr;
    uint64_t n = 0;
    if (stage == SIFT_CUDA_STAGE_CANDIDATES) {
        // per-octave regions, concatenated in octave order
        uint64_t total = 0;
        for (int o = 0; o < g.num_octaves; ++o) total += std::min<uint64_t>(c.oct[o].n_cand, e.cap_c[o]);
        *count = total;
        if (!out) return 0;
        uint64_t pos = 0;
        for (int o = 0; o < g.num_octaves && pos < capacity; ++o) {
            const uint64_t no = std::min<uint64_t>(c.oct[o].n_cand, e.cap_c[o]);
            const uint64_t m = std::min<uint64_t>(no, capacity - pos);
            if (m && cudaMemcpy((sift::Keypoint*)out + pos, e.d_cands.as<sift::Keypoint>() + e.cb[o],
                                m * sizeof(sift::Keypoint), cudaMemcpyDeviceToHost) != cudaSuccess)
                return sift::cuda_fail(cudaGetLastError(), "D2H stage");
            pos += m;
        }
        return 0;
    } else if (stage == SIFT_CUDA_STAGE_REFINED) {
        // the refined keypoints stay in their candidate slots with keep
        // flags; gathered here in slot order, octave after octave
        std::vector<sift::Keypoint> slots;
        std::vector<uint32_t> keep;
        uint64_t pos = 0, total = 0;
        for (int o = 0; o < g.num_octaves; ++o) {
            const uint64_t no = std::min<uint64_t>(c.oct[o].n_cand, e.cap_c[o]);
            slots.resize(no);
            keep.resize(no);
            if (no && (cudaMemcpy(slots.data(), e.d_refined_at.as<sift::Keypoint>() + e.cb[o],
                                  no * sizeof(sift::Keypoint), cudaMemcpyDeviceToHost) != cudaSuccess ||
                       cudaMemcpy(keep.data(), e.d_keep.as<uint32_t>() + e.cb[o], no * sizeof(uint32_t),
                                  cudaMemcpyDeviceToHost) != cudaSuccess))
                return sift::cuda_fail(cudaGetLastError(), "D2H stage");
            for (uint64_t i = 0; i < no; ++i) {
                if (!keep[i]) continue;
                if (out && pos < capacity) ((sift::Keypoint*)out)[pos++] = slots[i];
                ++total;
            }
        }
        *count = total;
        return 0;
    } else if (stage == SIFT_CUDA_STAGE_KEYPOINTS) {
        src = e.d_oriented.as<sift::Keypoint>();
        n = std::min<uint64_t>(c.n_oriented, e.cap_ori);
    } else if (stage == SIFT_CUDA_STAGE_DESCRIPTORS) {
        const uint64_t nd = std::min<uint64_t>(c.n_oriented, e.cap_ori) * sift::kDescLen;
        *count = nd;
        if (out && nd) {
            // after a host call the first descriptors are in the export buffer only
            const uint64_t m = std::min<uint64_t>(nd, capacity);
            const uint64_t on_host = std::min<uint64_t>((uint64_t)e.desc_on_host * sift::kDescLen, m);
            if (on_host) std::memcpy(out, e.hx_desc(), on_host * sizeof(float));
            if (m > on_host && cudaMemcpy((float*)out + on_host, e.d_desc.as<float>() + on_host,
                                          (m - on_host) * sizeof(float), cudaMemcpyDeviceToHost) != cudaSuccess)
                return sift::cuda_fail(cudaGetLastError(), "D2H stage");
        }
        return 0;
    } else {
        return sift::fail(SIFT_CUDA_ERR_INVALID_ARGUMENT, "unknown stage");
    }
    *count = n;
    if (out && n) {
        uint64_t m = std::min<uint64_t>(n, capacity);
        if (cudaMemcpy(out, src, m * sizeof(sift::Keypoint), cudaMemcpyDeviceToHost) != cudaSuccess)
            return sift::cuda_fail(cudaGetLastError(), "D2H stage");
    }
    return 0;
}

}  // extern "C"
