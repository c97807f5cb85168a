/*
 * sift_cuda.h — C ABI of libsiftcuda.so, the GB300 (sm_103a) SIFT engine.
 *
 * This is the boundary a `SiftBackend::Cuda` arm of the reference crate binds
 * through a thin `extern "C"` FFI crate. Each entry point names the reference
 * interface it replaces (stevel705/sift-wgpu, paths relative to the crate).
 *
 * Conventions
 *  - All entry points return 0 (SIFT_CUDA_OK) on success and a non-zero
 *    SiftCudaStatus on failure; sift_cuda_last_error() then returns a message
 *    for the calling thread (the reference returns Err(String),
 *    src/sift.rs:1244-1248). There is no CPU fallback.
 *  - Images are 8-bit grayscale, row-major, `stride` bytes between rows
 *    (stride >= width), the layout of `img.to_luma8().into_raw()`
 *    (src/sift.rs:1256-1258) when stride == width.
 *  - Keypoints and descriptors come back in the order of the reference CPU
 *    path: (octave, layer, y, x) of the detected extremum, then orientation
 *    peaks in histogram-bin order (src/sift.rs:510-603, 605-726).
 *  - An engine is not thread-safe: one thread at a time per engine.
 */
#ifndef SIFT_CUDA_H
#define SIFT_CUDA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SIFT_CUDA_DESCRIPTOR_LEN 128 /* 4x4x8, src/sift.rs:28-29 */

typedef enum {
    SIFT_CUDA_OK = 0,
    SIFT_CUDA_ERR_INVALID_ARGUMENT = 1,
    SIFT_CUDA_ERR_CUDA = 2,
    SIFT_CUDA_ERR_OUT_OF_MEMORY = 3,
    SIFT_CUDA_ERR_CAPACITY = 4, /* an internal list overflowed; never returned
                                   after the automatic retry with larger lists */
    SIFT_CUDA_ERR_NO_DEVICE = 5,
    SIFT_CUDA_ERR_UNSUPPORTED = 6
} SiftCudaStatus;

/* Sift's public fields (src/sift.rs:36-45). contrast_threshold is stored
 * already divided by num_intervals, exactly as Sift::new / Sift::default store
 * it (src/sift.rs:55,76); use sift_cuda_params_new to build it from the
 * undivided value. image_border_width is the private border (5,
 * src/sift.rs:17). */
typedef struct {
    float sigma;
    uint32_t num_octaves;
    uint32_t num_intervals;
    float assumed_blur;
    float contrast_threshold;
    float edge_threshold;
    uint32_t image_border_width;
} SiftCudaParams;

/* KeyPoint (src/keypoints.rs:2-10) as a C struct, 28 bytes. x, y in
 * full-resolution pixels, size = sigma (not diameter), angle in radians in
 * (-pi, pi], response = interpolated DoG value, octave/layer as the CPU path
 * sets them. */
typedef struct {
    float x, y, size, angle, response;
    int32_t octave, layer;
} SiftCudaKeypoint;

/* Library-owned result of one image: n keypoints and n x 128 descriptors
 * (desc == NULL for keypoint-only detection). Free with
 * sift_cuda_result_free. */
typedef struct {
    uint32_t n;
    SiftCudaKeypoint* kps;
    float* desc;
} SiftCudaResult;

/* Pyramid storage of the Gaussian levels in device memory. Levels of the
 * reference-compatible pyramid hold u8 integers, so every mode is exact.
 * Each level has a u8 plane, from which the detection forms DoG in f32 where
 * it reads it (no DoG plane is stored). U8 stores nothing else: orientation
 * and descriptors read v / 255 from the u8 planes through the IEEE quotient
 * table. F32 and F16 also store every level in that type (4 and 2 more bytes
 * per pixel), which orientation and descriptors then read. U8 is the default
 * (sift_cuda_options_default): the smallest footprint and, measured on a
 * GB300, the fastest of the three; all three give the same output. */
typedef enum {
    SIFT_CUDA_STORAGE_F32 = 0, /* u8 planes + levels stored as f32 (v / 255) */
    SIFT_CUDA_STORAGE_F16 = 1, /* u8 planes + levels stored as f16 (v) */
    SIFT_CUDA_STORAGE_U8 = 2   /* u8 planes only */
} SiftCudaStorage;

typedef struct {
    int32_t device;          /* CUDA device ordinal */
    int32_t storage;         /* SiftCudaStorage (default SIFT_CUDA_STORAGE_U8) */
    int32_t level_tile_rows; /* rows of the fused level kernel's tiles: 0 (default: 64), 64 or 32;
                                the output is the same (the batched form always uses 64) */
    uint32_t reserved[5];
} SiftCudaOptions;

typedef struct SiftCudaEngine SiftCudaEngine;

/* ---- parameters ---------------------------------------------------------- */

/* Sift::default() (src/sift.rs:47-59). */
void sift_cuda_params_default(SiftCudaParams* out);
/* Sift::new(sigma, num_octaves, num_intervals, assumed_blur,
 * contrast_threshold, edge_threshold) (src/sift.rs:63-80): stores
 * contrast_threshold / num_intervals. */
void sift_cuda_params_new(SiftCudaParams* out, float sigma, uint32_t num_octaves,
                          uint32_t num_intervals, float assumed_blur,
                          float contrast_threshold, float edge_threshold);
void sift_cuda_options_default(SiftCudaOptions* out);

/* ---- engine lifetime ----------------------------------------------------- */

/* Creates an engine bound to one GPU: stream, device arenas (grown on
 * demand and kept resident across calls) and weight tables. Replaces the
 * per-call GPU context construction of the GPU arms (src/sift.rs:1269-1285,
 * 1314-1329) with one long-lived context. opts may be NULL. */
int sift_cuda_create(const SiftCudaParams* params, const SiftCudaOptions* opts,
                     SiftCudaEngine** out);
void sift_cuda_destroy(SiftCudaEngine* engine);

/* ---- the drop-in call ---------------------------------------------------- */

/* Sift::detect_and_compute_with_backend(img, SiftBackend::Cuda)
 * (src/sift.rs:1244-1355) for an 8-bit grayscale host image: same keypoints,
 * order and 128-float descriptors as detect_and_compute_cpu
 * (src/sift.rs:1200-1240). The image is copied to the device inside the call;
 * results are copied back into library-owned host arrays. */
int sift_cuda_detect_and_compute(SiftCudaEngine* engine, const uint8_t* img, uint32_t width,
                                 uint32_t height, uint32_t stride, SiftCudaResult* out);

/* The same call with zero-copy results: out->kps and out->desc point into
 * pinned host buffers owned by the engine, valid until the next call on the
 * engine or sift_cuda_destroy; do not pass them to sift_cuda_result_free. The
 * form an FFI wrapper uses when it copies into its own containers anyway (the
 * Rust arm builds Vec<KeyPoint> / Vec<Vec<f32>>, src/sift.rs:1288-1291). */
int sift_cuda_detect_and_compute_view(SiftCudaEngine* engine, const uint8_t* img, uint32_t width,
                                      uint32_t height, uint32_t stride, SiftCudaResult* out);

/* Sift::detect (src/sift.rs:846-886): keypoints with orientation, no
 * descriptors (out->desc == NULL). */
int sift_cuda_detect(SiftCudaEngine* engine, const uint8_t* img, uint32_t width, uint32_t height,
                     uint32_t stride, SiftCudaResult* out);

void sift_cuda_result_free(SiftCudaResult* result);

/* ---- colour input ----------------------------------------------------------- */

/* Pixel formats of sift_cuda_detect_and_compute_pixels. The conversion to
 * 8-bit luma runs on the device:
 *   GRAY8          as sift_cuda_detect_and_compute
 *   RGB8, RGBA8    DynamicImage::to_luma8 (src/sift.rs:1202, 1256; image 0.25.6:
 *                  (2126 r + 7152 g + 722 b) / 10000, integer, alpha ignored)
 *   RGBA8_CANVAS   the WASM entry's img_from_raw (src/wasm.rs:79-104):
 *                  0.299 r + 0.587 g + 0.114 b in f32, truncated to u8 */
enum {
    SIFT_CUDA_PIXELS_GRAY8 = 0,
    SIFT_CUDA_PIXELS_RGB8 = 1,
    SIFT_CUDA_PIXELS_RGBA8 = 2,
    SIFT_CUDA_PIXELS_RGBA8_CANVAS = 3
};

/* detect_and_compute_with_backend on a colour image (`stride` in bytes,
 * >= width x channels): the host->device copy moves the colour bytes and the
 * luma conversion is one more kernel before the pipeline. */
int sift_cuda_detect_and_compute_pixels(SiftCudaEngine* engine, const uint8_t* pixels, uint32_t width,
                                        uint32_t height, uint32_t stride, int32_t format,
                                        SiftCudaResult* out);
/* The conversion alone, device to device, asynchronous on `stream`
 * (a cudaStream_t; NULL = default stream). */
int sift_cuda_to_luma(const uint8_t* d_pixels, uint32_t width, uint32_t height, uint32_t stride,
                      int32_t format, uint8_t* d_out, uint32_t out_stride, void* stream);

/* Message of the last failure on the calling thread ("" if none). */
const char* sift_cuda_last_error(void);

/* ---- device-resident form ------------------------------------------------ */

/* Runs the whole pipeline on an image already in device memory, on the
 * engine's stream, without copying results back; the outputs stay in the
 * engine's device arena until the next call. `d_count` receives a device
 * pointer to the keypoint count, d_kps / d_desc device pointers to the arrays.
 * Returns without synchronising; call sift_cuda_synchronize before reading.
 * Replaces the readback-free part of GpuSiftV2::detect
 * (src/gpu_sift_v2.rs:789-858). */
int sift_cuda_run_device(SiftCudaEngine* engine, const uint8_t* d_img, uint32_t width,
                         uint32_t height, uint32_t stride, int with_descriptors);
int sift_cuda_device_outputs(SiftCudaEngine* engine, const uint32_t** d_count,
                             const SiftCudaKeypoint** d_kps, const float** d_desc);
int sift_cuda_synchronize(SiftCudaEngine* engine);
/* The engine's cudaStream_t, as void* (no CUDA types in this header). */
void* sift_cuda_stream(SiftCudaEngine* engine);

/* ---- introspection used by the parity tests -------------------------------- */

/* Stages of the last run, copied to host memory:
 *  SIFT_CUDA_STAGE_PYRAMID:    all Gaussian levels as u8, octave-major, then
 *                              level, row-major with stride = octave width;
 *                              element size 1.
 *  SIFT_CUDA_STAGE_CANDIDATES: find_scale_space_extrema output
 *                              (src/sift.rs:510-603), SiftCudaKeypoint each.
 *  SIFT_CUDA_STAGE_REFINED:    refine_and_filter_extrema output
 *                              (src/sift.rs:299-474), SiftCudaKeypoint each.
 *  SIFT_CUDA_STAGE_DOG:        all DoG levels as f32, octave-major, level,
 *                              row-major, formed on the device from the u8
 *                              level planes by the function the candidate
 *                              emission and refinement read DoG through.
 *  SIFT_CUDA_STAGE_KEYPOINTS:  the final keypoints, SiftCudaKeypoint each.
 *  SIFT_CUDA_STAGE_DESCRIPTORS: the final descriptors, 128 floats each
 *                              (count = keypoints x 128).
 * Writes at most `capacity` elements and the total count to *count. */
enum {
    SIFT_CUDA_STAGE_PYRAMID = 0,
    SIFT_CUDA_STAGE_CANDIDATES = 1,
    SIFT_CUDA_STAGE_REFINED = 2,
    SIFT_CUDA_STAGE_DOG = 3,
    SIFT_CUDA_STAGE_KEYPOINTS = 4,
    SIFT_CUDA_STAGE_DESCRIPTORS = 5
};
int sift_cuda_debug_stage(SiftCudaEngine* engine, int stage, void* out, uint64_t capacity,
                          uint64_t* count);

/* Device-side kernel launches of the last run (for launch accounting). */
uint32_t sift_cuda_last_launch_count(SiftCudaEngine* engine);

/* 1 if the last host call's run read the image where the caller keeps it (a
 * pageable host image, 16-byte aligned with a stride a multiple of 16, on a
 * device that reads pageable host memory coherently, e.g. a GB300 with its
 * Grace host), 0 if it read the engine's device copy. */
uint32_t sift_cuda_last_image_in_place(SiftCudaEngine* engine);

/* Per-stage device time accounting, the CUDA-event counterpart of the
 * reference's SIFT_PROFILE stage timers (src/gpu_sift_v2.rs:795-855). While
 * enabled, every run records events on the engine's stream at the stage
 * boundaries. sift_cuda_profile_read synchronises and returns the summed
 * milliseconds of the runs since the last read:
 *   [0] Gaussian pyramid + DoG, [1] extrema + refinement + compaction,
 *   [2] orientation, [3] descriptors. */
enum { SIFT_CUDA_PROFILE_STAGES = 4 };
int sift_cuda_profile_enable(SiftCudaEngine* engine, int enable);
int sift_cuda_profile_read(SiftCudaEngine* engine, float* stage_ms, uint32_t n_stages, uint32_t* runs);

/* ---- serving: continuous batching over resident engines ------------------ */

/* The serving and batching forms of SiftBackend::Cuda (no counterpart in the
 * reference, whose GPU arms build a context per call, src/sift.rs:1262-1291).
 * A server keeps one resident engine ("slot") per image size and in-flight
 * request, admits requests by the device footprint of their slot against
 * arena_bytes, and runs up to max_inflight of them concurrently on separate
 * streams; a request that arrives while others run starts as soon as a slot
 * of its size is idle or fits. One internal host thread issues all CUDA work.
 * Results are bit-identical to sift_cuda_detect_and_compute on the same image
 * and parameters, alone or in any mix. */
typedef struct SiftCudaServer SiftCudaServer;

typedef struct {
    int32_t device;
    int32_t storage;       /* SiftCudaStorage */
    uint64_t arena_bytes;  /* device bytes the slots may hold (default 40 GiB) */
    uint32_t max_inflight; /* requests on the device at once (default 8) */
    uint32_t autotune;     /* 1: time launch shapes on the first slot of each size */
    uint32_t reserved[4];
} SiftCudaServerOptions;

typedef struct {
    uint64_t ticket;             /* pass to sift_cuda_server_release */
    uint64_t tag;                /* the caller's tag from submit */
    int32_t status;              /* 0 or a SiftCudaStatus */
    uint32_t n;                  /* keypoints */
    const SiftCudaKeypoint* kps; /* valid until released */
    const float* desc;           /* n x 128, valid until released */
    double submit_s, start_s, done_s; /* steady-clock seconds */
} SiftCudaServed;

typedef struct {
    uint32_t slots, running, pending, reserved;
    uint64_t device_bytes, completed, reruns, evicted, max_pending;
} SiftCudaServerStats;

enum { SIFT_CUDA_SUBMIT_BORROW = 1 }; /* img stays valid and unchanged until polled: no copy */

void sift_cuda_server_options_default(SiftCudaServerOptions* out);
int sift_cuda_server_create(const SiftCudaParams* params, const SiftCudaServerOptions* opts,
                            SiftCudaServer** out);
/* Waits for the requests in flight, then frees everything. */
void sift_cuda_server_destroy(SiftCudaServer* server);
/* Queues one image (copied unless SIFT_CUDA_SUBMIT_BORROW); *ticket names it. */
int sift_cuda_server_submit(SiftCudaServer* server, const uint8_t* img, uint32_t width, uint32_t height,
                            uint32_t stride, uint64_t tag, uint32_t flags, uint64_t* ticket);
/* Next finished request: 1 and *out filled, 0 on timeout (timeout_us < 0
 * waits without limit, 0 does not wait). */
int sift_cuda_server_poll(SiftCudaServer* server, SiftCudaServed* out, int64_t timeout_us);
/* Gives the request's slot back; its kps/desc pointers become invalid. */
int sift_cuda_server_release(SiftCudaServer* server, uint64_t ticket);
/* Runs `count` concurrent requests of this image (untimed warm-up): creates
 * up to `count` slots of its size and captures their graphs. */
int sift_cuda_server_warm(SiftCudaServer* server, const uint8_t* img, uint32_t width, uint32_t height,
                          uint32_t stride, uint32_t count);
int sift_cuda_server_stats(SiftCudaServer* server, SiftCudaServerStats* out);
/* Launch shape chosen for a size by the autotuner: [fused blur radius limit,
 * orientation CTAs/SM, descriptor CTAs/SM]; returns 1 if tuned, 0 if default. */
int sift_cuda_server_tuning(SiftCudaServer* server, uint32_t width, uint32_t height, int32_t* knobs3);
/* The same with every knob: writes the first min(n_knobs, 4) of [fused blur
 * radius limit, fused level tile rows (64 or 32), orientation CTAs/SM,
 * descriptor CTAs/SM]; returns 1 if tuned, 0 if default. */
int sift_cuda_server_tuning_knobs(SiftCudaServer* server, uint32_t width, uint32_t height, int32_t* knobs,
                                  uint32_t n_knobs);
/* Device bytes a slot for a width x height image holds (admission estimate). */
uint64_t sift_cuda_footprint_bytes(const SiftCudaParams* params, int32_t storage, uint32_t width,
                                   uint32_t height);

/* Open-loop replay of a request trace: request i is due at start +
 * arrival_s and its latency runs from that due time until its result is in
 * host memory. server != NULL drives the server (images are borrowed: keep
 * them pinned for speed); server == NULL runs the plain path instead — one
 * synchronous sift_cuda_detect_and_compute_view per request, in arrival
 * order, on an engine per image size created from params/opts. */
typedef struct {
    const uint8_t* data;
    uint32_t width, height, stride, reserved;
} SiftCudaReplayImage;
typedef struct {
    double arrival_s;
    uint32_t image, reserved;
} SiftCudaReplayRequest;
typedef struct {
    double latency_s;
    uint32_t n;
    int32_t status;
} SiftCudaReplayResult;
int sift_cuda_replay(SiftCudaServer* server, const SiftCudaParams* params, const SiftCudaOptions* opts,
                     const SiftCudaReplayImage* images, uint32_t n_images, const SiftCudaReplayRequest* reqs,
                     uint32_t n_reqs, SiftCudaReplayResult* results, double* wall_s);

/* ---- batched form: one run over many images ------------------------------ */

/* detect_and_compute_with_backend (src/sift.rs:1244-1355) on a batch of 8-bit
 * grayscale images of any sizes in one run (no counterpart in the reference,
 * whose GPU arms take one image per call). Each stage of the hot path is one
 * launch over the flattened work of every image: the pyramid one launch per
 * (octave, level) over the tiles of that octave of all images, then
 * extrema, candidate scan, emission, refinement, orientation, oriented
 * keypoints and descriptors one launch each over all (image, octave)
 * entries; the run is captured once per batch geometry as a CUDA graph. Every
 * image's keypoints and descriptors are those of sift_cuda_detect_and_compute
 * on it, bit for bit, in the same order. The batch keeps its levels as u8
 * planes (opts->storage must be SIFT_CUDA_STORAGE_U8). */
typedef struct {
    const uint8_t* data;
    uint32_t width, height, stride, reserved;
} SiftCudaImage;

typedef struct {
    uint32_t n_images, total;
    const uint32_t* offsets;     /* n_images + 1: image i's keypoints are [offsets[i], offsets[i + 1]) */
    const SiftCudaKeypoint* kps; /* total keypoints, image after image */
    const float* desc;           /* total x 128 */
    uint32_t launches;           /* kernel launches of the run */
    float device_ms;             /* device time of the run (from its first kernel) */
    uint32_t images_in_place;    /* 1: the run read the images from the caller's buffers (a device
                                    that reads pageable host memory, every image 16-byte aligned
                                    with a stride a multiple of 16); 0: from a device copy */
} SiftCudaBatchResult;

typedef struct SiftCudaBatch SiftCudaBatch;

int sift_cuda_batch_create(const SiftCudaParams* params, const SiftCudaOptions* opts, SiftCudaBatch** out);
void sift_cuda_batch_destroy(SiftCudaBatch* batch);
/* Runs the batch and synchronises. The result's arrays are mapped pinned host
 * buffers owned by the batch object (the run writes them from the device),
 * valid until its next call or destroy. */
int sift_cuda_batch_detect_and_compute(SiftCudaBatch* batch, const SiftCudaImage* images, uint32_t n,
                                       SiftCudaBatchResult* out);

/* ---- descriptor matching ------------------------------------------------ */

/* The nearest and second-nearest train descriptor of each query descriptor
 * by Euclidean distance (brute force, f32): the input of Lowe's ratio test.
 * Not in the reference crate; it consumes the 128-float descriptors that
 * detect_and_compute returns. Ties go to the lower train index. */
typedef struct {
    int32_t train_idx;      /* nearest train descriptor, -1 if n_train == 0 */
    float distance;         /* its Euclidean distance (INFINITY if none) */
    int32_t second_idx;     /* second nearest, -1 if n_train < 2 */
    float second_distance;
} SiftCudaMatch;

/* Host arrays: query n_query x 128 floats, train n_train x 128 floats, out
 * n_query entries; runs on the engine's stream and synchronises. */
int sift_cuda_match(SiftCudaEngine* engine, const float* query, uint32_t n_query, const float* train,
                    uint32_t n_train, SiftCudaMatch* out);
/* Device form, asynchronous on `stream` (a cudaStream_t; NULL = default):
 * d_query and d_train 16-byte aligned, d_scratch at least
 * sift_cuda_match_scratch_bytes(n_query, n_train) bytes of device memory. */
size_t sift_cuda_match_scratch_bytes(uint32_t n_query, uint32_t n_train);
int sift_cuda_match_device(const float* d_query, uint32_t n_query, const float* d_train, uint32_t n_train,
                           SiftCudaMatch* d_out, void* d_scratch, void* stream);

/* ---- drawing ---------------------------------------------------------------- */

/* draw_keypoints_to_image (src/lib.rs:69-116): the grey image as RGB with,
 * for every keypoint, a filled circle of radius 6 at (x as i32, y as i32), the
 * orientation line from (x, y) to (x + 6 cos angle, y + 6 sin angle) and a
 * filled circle of radius 1, in colour (r, g, b) (imageproc 0.25.0
 * draw_filled_circle_mut / draw_line_segment_mut, restated). Host buffers:
 * gray width x height with `stride` bytes per row, rgb_out width x height x 3
 * with out_stride >= 3 * width bytes per row. Synchronous. */
int sift_cuda_draw_keypoints(SiftCudaEngine* engine, const uint8_t* gray, uint32_t width, uint32_t height,
                             uint32_t stride, const SiftCudaKeypoint* kps, uint32_t n, uint8_t r, uint8_t g,
                             uint8_t b, uint8_t* rgb_out, uint32_t out_stride);

/* ---- blur without allocation ---------------------------------------------- */

/* Gaussian blur of a u8 image in device memory into a caller-owned device
 * buffer, with the arithmetic of every blur of the pyramid (imageproc 0.25.0
 * gaussian_blur_f32 on u8: radius ceil(2 sigma), clamp-to-edge, horizontal
 * then vertical pass, each truncated to u8). This entry point has no
 * counterpart in the reference; it serves callers that must not allocate
 * device memory on their path (a process whose memory pool has reserved the
 * free device memory, or a loop that cannot take cudaFree's device-wide
 * synchronisation). The horizontal pass's intermediate lives in a fixed
 * 16 MiB device array inside this library, so the call allocates nothing.
 *  - Limits: width <= 8192, align16(width) * height <= 16 MiB (4096 x 4096
 *    fits), ceil(2 sigma) <= 64; beyond them SIFT_CUDA_ERR_UNSUPPORTED and
 *    nothing runs. d_dst may equal d_src.
 *  - The first call on a device looks the array's address up (and may make
 *    the runtime load this library's device code there): make it before any
 *    stream capture begins. The address is kept for the life of the process:
 *    do not use this entry point after a cudaDeviceReset of that device (the
 *    module may reload elsewhere).
 *  - Calls share the array: calls that can overlap on the device (different
 *    streams, unordered threads) race and corrupt each other's output.
 *  - Asynchronous on `stream` (a cudaStream_t; NULL = the default stream). */
int sift_cuda_gaussian_blur_u8_noalloc(const uint8_t* d_src, uint32_t width, uint32_t height,
                                       uint32_t src_stride, uint8_t* d_dst, uint32_t dst_stride,
                                       float sigma, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* SIFT_CUDA_H */
