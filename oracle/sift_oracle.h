/*
 * sift_oracle.h — C ABI of the CPU oracle.
 *
 * TEST INFRASTRUCTURE ONLY. This library is a CPU restatement of the reference
 * CPU SIFT path (src/sift.rs of stevel705/sift-wgpu, plus the two third-party
 * routines it calls: imageproc 0.25.0 gaussian_blur_f32 and image 0.25.6
 * resize_exact(Lanczos3)). It is the checker the CUDA path is compared against
 * and the CPU baseline that is timed beside it. Nothing in the product links or
 * calls it.
 *
 * Parity status: the leaf routines (3x3 Cramer solve, bilinear sampling) are
 * pinned by the reference's own known-answer tests (src/sift.rs:1424-1525) and
 * the end-to-end properties of tests/integration_test.rs. The blur and the
 * Lanczos3 resize live in crates that are not vendored in the reference, so
 * their restatement is "parity unpinned" (published algorithm, no golden
 * vectors); the switches in OracleBlurModel isolate the uncertain choices.
 */
#ifndef SIFT_ORACLE_H
#define SIFT_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Same layout as SiftCudaParams in include/sift_cuda.h. contrast_threshold is
 * already divided by num_intervals, as Sift::new / Sift::default store it
 * (src/sift.rs:55,76). */
typedef struct {
    float sigma;
    uint32_t num_octaves;
    uint32_t num_intervals;
    float assumed_blur;
    float contrast_threshold;
    float edge_threshold;
    uint32_t image_border_width;
} OracleParams;

/* Same layout as SiftCudaKeypoint (KeyPoint, src/keypoints.rs:2-10). */
typedef struct {
    float x, y, size, angle, response;
    int32_t octave, layer;
} OracleKeypoint;

typedef struct {
    uint32_t n;
    OracleKeypoint* kps;
    float* desc; /* n x 128 */
} OracleResult;

/* Intermediate stages of one run, for stage-wise parity tests. */
typedef struct {
    uint32_t num_octaves, levels_per_octave; /* levels = S + 3 */
    uint32_t* oct_w;                          /* [num_octaves] */
    uint32_t* oct_h;
    uint8_t* pyramid;      /* all Gaussian levels, octave-major, level, row-major */
    uint64_t pyramid_bytes;
    uint32_t n_candidates;
    OracleKeypoint* candidates; /* find_scale_space_extrema output */
    uint32_t n_refined;
    OracleKeypoint* refined;    /* refine_and_filter_extrema output */
    OracleResult result;        /* oriented keypoints + descriptors */
} OracleStages;

/* Switches for the parts restated from crates absent from the reference. */
typedef struct {
    int blur_radius_factor_x100; /* kernel radius = ceil(f * sigma); imageproc: 200 */
    int blur_normalize;          /* 0: raw Gaussian samples (imageproc), 1: sum to 1 */
    int blur_round;              /* 0: truncate f32->u8 (imageproc Clamp), 1: round */
} OracleBlurModel;

void oracle_default_params(OracleParams* p);
/* Sift::new(sigma, octaves, intervals, assumed_blur, contrast, edge): divides
 * contrast by intervals (src/sift.rs:63-80). */
void oracle_new_params(OracleParams* p, float sigma, uint32_t num_octaves, uint32_t num_intervals,
                       float assumed_blur, float contrast_threshold, float edge_threshold);

void oracle_get_blur_model(OracleBlurModel* m);
void oracle_set_blur_model(const OracleBlurModel* m);

/* detect_and_compute_cpu (src/sift.rs:1200-1240). threads: worker threads for
 * the axes rayon parallelises in the reference (0 = all cores, 1 = serial).
 * Returns 0 on success. */
int oracle_detect_and_compute(const OracleParams* p, const uint8_t* img, uint32_t w, uint32_t h,
                              uint32_t stride, int threads, OracleResult* out);
/* Sift::detect (src/sift.rs:846-886): keypoints only, desc == NULL. */
int oracle_detect(const OracleParams* p, const uint8_t* img, uint32_t w, uint32_t h,
                  uint32_t stride, int threads, OracleResult* out);
void oracle_result_free(OracleResult* r);

int oracle_stages(const OracleParams* p, const uint8_t* img, uint32_t w, uint32_t h,
                  uint32_t stride, int threads, OracleStages* out);
void oracle_stages_free(OracleStages* s);

/* Leaf routines, exposed for the reference's known-answer tests. */
/* gaussian_blur_f32 on a u8 image (imageproc). */
void oracle_gaussian_blur_u8(const uint8_t* in, uint32_t w, uint32_t h, float sigma, uint8_t* out);
/* The 1-D kernel gaussian_blur_f32 builds; returns its length (2r+1), writes
 * up to cap weights. */
int oracle_gaussian_kernel(float sigma, float* out, int cap);
/* resize_exact(Lanczos3) on a u8 image (image crate). */
void oracle_resize_lanczos3_u8(const uint8_t* in, uint32_t w, uint32_t h, uint32_t nw, uint32_t nh,
                               uint8_t* out);
/* solve_linear_system (src/sift.rs:478-503): returns 1 and writes x on
 * success, 0 when |det| < 1e-10. a is row-major 3x3. */
int oracle_solve3(const float* a, const float* b, float* x);
/* get_gauss_pixel_bilinear (src/sift.rs:238-266). */
float oracle_bilinear(const uint8_t* img, uint32_t w, uint32_t h, float x, float y);
/* The Gaussian blur sigmas of the pyramid (src/sift.rs:129-177): writes
 * sigma_base then, per octave, the S+2 increments (0 when the level is a
 * copy). Returns the number of floats written. */
int oracle_blur_sigmas(const OracleParams* p, float* out, int cap);

#ifdef __cplusplus
}
#endif
#endif
