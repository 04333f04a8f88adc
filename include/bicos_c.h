/*
 * bicos_gb300 -- C ABI of the GB300-native BICOS matcher (sm_103a).
 *
 * This is the drop-in boundary for libBICOS's matching path.  Every entry
 * point takes plain pointers, sizes and POD structs; images are device
 * resident, one pitched 2-D image per frame, exactly as the reference's
 * cv::cuda::GpuMat inputs.  Work is enqueued on the caller's stream and the
 * call returns without waiting for it (the reference returned after its
 * implicit synchronisation; call cudaStreamSynchronize to get that).
 *
 * Reference interfaces replaced (paths inside libBICOS 2.2.0):
 *   bicos_match_v1                 BICOS::match, include/match.hpp:31-41,
 *                                  src/lib.cpp:31-49, src/impl/cuda.cu.in:233-292
 *   bicos_descriptor_transform_v1  transform_{limited,full}_kernel,
 *                                  include/impl/cuda/descriptor_transform.cuh:30-149
 *   bicos_search_v1                bicos_kernel(_smem),
 *                                  include/impl/cuda/bicos.cuh:77-176
 *   bicos_agree_v1                 agree_kernel, include/impl/cuda/agree.cuh:110-159
 *   bicos_agree_subpixel_v1        agree_subpixel_kernel,
 *                                  include/impl/cuda/agree.cuh:161-259
 *   bicos_config_default           BICOS::Config defaults, include/common.hpp:73-82
 *   bicos_last_error               BICOS::Exception::what(), src/exception.cpp:23-27
 *   bicos_reproject_v1             bicos-cli's cv::reprojectImageTo3D step,
 *                                  src/cli.cpp:228-250
 *   bicos_png_unfilter             the PNG decoding bicos-cli gets from cv::imread,
 *                                  src/fileutils.cpp:61-83 (host utility)
 * Extensions without a reference counterpart: bicos_match_host_v1 (host
 * buffers, pybicos's path), bicos_search_bits_v1, bicos_search_noalloc_v1,
 * the learned-form, MLP and batch entry points.
 *
 * Error behaviour: every entry point returns a bicos_status.  Messages match
 * the reference's exception texts ("need at least two images", "bad input
 * depths, only CV_8UC1 and CV_16UC1 are supported", "input stacks too large,
 * would require N bits") and are read back with bicos_last_error(), which is
 * per thread.  BICOS_ERR_INVALID_ARGUMENT corresponds to the reference's
 * std::invalid_argument, BICOS_ERR_EXCEPTION to BICOS::Exception.
 */
#ifndef BICOS_GB300_C_H
#define BICOS_GB300_C_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* a cudaStream_t; 0 is the legacy default stream */
typedef struct CUstream_st* bicos_stream_t;

/* element types: OpenCV's single-channel type codes (CV_8UC1 ...) */
enum {
    BICOS_8U = 0,
    BICOS_16U = 2,
    BICOS_16S = 3,
    BICOS_32F = 5,
    BICOS_64F = 6,
    BICOS_32FC3 = 21 /* three float channels per pixel (point clouds) */
};

typedef enum bicos_status {
    BICOS_OK = 0,
    BICOS_ERR_EXCEPTION = 1,        /* BICOS::Exception */
    BICOS_ERR_INVALID_ARGUMENT = 2, /* std::invalid_argument */
    BICOS_ERR_CUDA = 3              /* a CUDA runtime error (BICOS::Exception in the reference) */
} bicos_status;

/* a pitched device image (the layout of cv::cuda::GpuMat's header) */
typedef struct bicos_image {
    void* data;
    size_t step; /* bytes between rows */
    int32_t rows;
    int32_t cols;
    int32_t type; /* BICOS_8U ... */
    int32_t reserved;
} bicos_image;

/* descriptor transform modes, BICOS::TransformMode */
enum { BICOS_MODE_LIMITED = 0, BICOS_MODE_FULL = 1 };
/* NCC precision, BICOS::Precision */
enum { BICOS_PRECISION_SINGLE = 0, BICOS_PRECISION_DOUBLE = 1 };
/* search variant, BICOS::Variant::{NoDuplicates, Consistency} */
enum { BICOS_VARIANT_NODUPLICATES = 0, BICOS_VARIANT_CONSISTENCY = 1 };
/* search flags, include/impl/common.hpp:46-47 */
enum { BICOS_FLAG_NODUPES = 1, BICOS_FLAG_CONSISTENCY = 2 };

/* BICOS::Config, field for field; std::optional<float> is (has_x, x) */
typedef struct bicos_config {
    int32_t has_threshold;
    float nxcorr_threshold;   /* default 0.5 */
    int32_t has_subpixel_step;
    float subpixel_step;      /* default none */
    int32_t has_min_variance;
    float min_variance;       /* default none; per frame, scaled by n internally */
    int32_t mode;             /* default BICOS_MODE_LIMITED */
    int32_t precision;        /* default BICOS_PRECISION_SINGLE */
    int32_t variant;          /* default BICOS_VARIANT_NODUPLICATES */
    int32_t max_lr_diff;      /* Consistency only, default 1 */
    int32_t no_dupes;         /* Consistency only, default 0 */
    int32_t max_bits;         /* descriptor width limit: 256 as the reference;
                                 up to 512 accepts FULL stacks of n <= 23 (extension) */
    int32_t nxcorr_form;      /* BICOS_NXCORR_REFERENCE (default), BICOS_NXCORR_MOMENTS or
                                 BICOS_NXCORR_LEARNED */
} bicos_config;

/* NCC forms.  REFERENCE: the reference's two-pass NCC, bit-identical
 * results.  MOMENTS (extension, no counterpart in the reference): the
 * correlation from exact integer moments, with the Sxy band formed on the
 * tensor cores and the subpixel interpolant left unrounded, so the sweep's
 * correlation is a closed-form function of the position; FP64 (precision
 * double) or FP32 evaluates only the final polynomials and ratio.  Results
 * differ from the reference's by the rounding of its interpolants.  The
 * moments are exact integers for every input: 8-bit samples and 16-bit
 * samples below 4096 take the tensor-core band, tiles holding a larger
 * 16-bit sample the SIMT sums. */
enum { BICOS_NXCORR_REFERENCE = 0, BICOS_NXCORR_MOMENTS = 1, BICOS_NXCORR_LEARNED = 2 };
/* LEARNED (extension, no counterpart in the reference; subpixel runs only,
 * other runs take the reference form): a small network proposes each
 * match's subpixel offset x from the correlations at the integer disparities
 * d-2..d+2 and the per-pixel variances; one NCC evaluation in the
 * reference's arithmetic (its rounded interpolants, its precision) at x
 * accepts the proposal when rho(x) >= rho(d) - 0.002, giving d - x and
 * rho(x) exactly as the sweep would for that x; every other pixel takes the
 * reference sweep with the configured step.  Needs an installed model
 * (bicos_learned_model_v1; the library carries a trained one). */

/* Fills the reference defaults (include/common.hpp:73-82). */
bicos_status bicos_config_default(bicos_config* cfg);

/* Per-thread text of the last error. */
const char* bicos_last_error(void);

/* Output element types match() produces for a configuration:
 * disparity BICOS_16S (no threshold or no step) or BICOS_32F (step);
 * corrmap BICOS_32F / BICOS_64F by precision, or -1 when none is made. */
bicos_status bicos_output_types(const bicos_config* cfg, int32_t* disparity_type,
                                int32_t* corrmap_type);

/* Descriptor width in 32-bit words for n frames in a mode (1, 2, 4, 8; 12
 * or 16 past 256 bits when max_bits allows), or -1 when too large. */
int32_t bicos_descriptor_words(uint32_t n, int32_t mode, int32_t max_bits);

/*
 * The whole matching path: BICOS::match(stack0, stack1, disparity, cfg,
 * corrmap, stream).
 *   stack0, stack1  n device images each, all of one size and of type
 *                   BICOS_8U or BICOS_16U
 *   disparity       caller-allocated device image of the size of the stack
 *                   and of the type bicos_output_types() reports
 *   corrmap         NULL, or a device image likewise; pixels that get no
 *                   correlation are NaN
 * Scratch (descriptors, raw disparities) comes from a per-device cache that
 * grows on demand and is reused across calls; calls on several streams are
 * ordered by an event.  bicos_release_scratch() frees it.
 */
bicos_status bicos_match_v1(const bicos_image* stack0, const bicos_image* stack1, uint32_t n,
                            bicos_image* disparity, bicos_image* corrmap,
                            const bicos_config* cfg, bicos_stream_t stream);

/*
 * bicos_match_v1 over HOST buffers, synchronous: the path pybicos.match
 * takes (src/pybicos.cpp:102-119 uploads each image, matches, downloads).
 * frames0/frames1 are n host pointers to rows x cols images of `type` with
 * row step host_step; disparity (and corrmap, may be NULL) are host buffers
 * of the types bicos_output_types() reports.  Device copies live in a
 * per-device staging cache; returns after the results are in host memory.
 */
bicos_status bicos_match_host_v1(const void* const* frames0, const void* const* frames1, uint32_t n,
                                 int32_t rows, int32_t cols, int32_t type, size_t host_step,
                                 void* disparity, size_t disparity_step, void* corrmap,
                                 size_t corrmap_step, const bicos_config* cfg,
                                 bicos_stream_t stream);

/* Frees this device's cached scratch memory (waits for its last use). */
bicos_status bicos_release_scratch(void);

/*
 * Stage entry points (kernel-level interfaces of the reference).
 * Descriptors are dense [rows][cols][nwords] uint32 arrays in device
 * memory, bit i of a descriptor in word i/32, bit i%32.
 */
bicos_status bicos_descriptor_transform_v1(const bicos_image* stack, uint32_t n, int32_t mode,
                                           uint32_t nwords, uint32_t* descriptors,
                                           bicos_stream_t stream);

/* Row-wise Hamming arg-min of desc0 against desc1 with flags
 * (BICOS_FLAG_*; 0 = plain first minimum).  Writes int16 disparities
 * col0 - col1 (INT16_MIN = invalid) to `disparity` (BICOS_16S). */
bicos_status bicos_search_v1(const uint32_t* desc0, const uint32_t* desc1, int32_t rows,
                             int32_t cols, uint32_t nwords, int32_t flags, int32_t max_lr_diff,
                             bicos_image* disparity, bicos_stream_t stream);

/* bicos_search_v1 for descriptors that use only bit positions
 * 0..bits-1 (1 <= bits <= 32*nwords; LSB-first, bit i in word i/32): the
 * positions from `bits` on must be zero, as bicos_descriptor_transform_v1
 * leaves them.  No counterpart in the reference, whose descriptor type
 * fixes the width.  With bits <= 32*nwords - 2 (every descriptor the
 * transform writes) the tensor-core search carries each candidate's column
 * in the two unused top positions, so the product itself is the
 * first-minimum key.  Outputs equal bicos_search_v1's. */
bicos_status bicos_search_bits_v1(const uint32_t* desc0, const uint32_t* desc1, int32_t rows,
                                  int32_t cols, uint32_t nwords, int32_t bits, int32_t flags,
                                  int32_t max_lr_diff, bicos_image* disparity,
                                  bicos_stream_t stream);

/*
 * bicos_search_v1 without any device allocation.  No counterpart in the
 * reference: for callers that cannot call cudaMalloc while they run (a
 * real-time loop with a fixed memory plan, a host framework that owns all
 * device memory and forbids allocation in its callbacks, code that must not
 * meet an allocation failure or an allocator synchronisation mid-pipeline).
 * The consistency flags need scratch for the forward and backward best
 * columns; here it is a fixed 32 MiB device array inside the library
 * (limit rows * cols <= 4194304 pixels, larger sizes fail with
 * BICOS_ERR_INVALID_ARGUMENT), held by every GPU that loads it until the
 * process exits.  The first call on a device looks up the array's device
 * address (cudaGetSymbolAddress) with that device current, which under
 * lazy module loading also loads the array: make one consistency call at
 * initialisation, outside any stream capture (a failed lookup is retried on
 * the next call).  All calls share the array: calls that
 * overlap on the GPU race, so serialise them.  Without the consistency flag
 * no scratch is used.  Outputs equal bicos_search_v1's.
 */
bicos_status bicos_search_noalloc_v1(const uint32_t* desc0, const uint32_t* desc1, int32_t rows,
                                     int32_t cols, uint32_t nwords, int32_t flags,
                                     int32_t max_lr_diff, bicos_image* disparity,
                                     bicos_stream_t stream);

/*
 * Point cloud of a disparity map: cv::reprojectImageTo3D(disparity, points,
 * Q, false, CV_32F) as bicos-cli runs it after the match (src/cli.cpp:
 * 228-250).  Every pixel (x, y) with disparity d becomes
 * (X/W, Y/W, Z/W) with [X Y Z W]^T = Q [x y d 1]^T (W = 0 gives (0, 0, 0));
 * invalid disparities are reprojected too, as values (INT16_MIN; NaN
 * propagates) and left for the point-cloud writer to skip.
 *   disparity  BICOS_16S or BICOS_32F device image (the match's output)
 *   q          16 doubles, Q row-major (host memory, read during the call)
 *   points     BICOS_32FC3 device image of the disparity's size
 * Arithmetic in FP32 (fused sums of the Q terms).
 */
bicos_status bicos_reproject_v1(const bicos_image* disparity, const double* q, bicos_image* points,
                                bicos_stream_t stream);

/*
 * bicos_match_v1 plus the point cloud of its disparity in the same pass:
 * the match bicos-cli runs followed by its cv::reprojectImageTo3D step
 * (src/cli.cpp:188-194, 228-250).  Arguments and outputs as
 * bicos_match_v1; q and points as bicos_reproject_v1, whose points this
 * writes bit for bit.  With a threshold, the agreement kernels (of every
 * NCC form) write each pixel's point as they write its disparity (no
 * second pass over HBM); without one, the reprojection pass runs after the
 * search on `stream`.
 */
bicos_status bicos_match_points_v1(const bicos_image* stack0, const bicos_image* stack1, uint32_t n,
                                   bicos_image* disparity, bicos_image* corrmap, const bicos_config* cfg,
                                   const double* q, bicos_image* points, bicos_stream_t stream);

/* Host utility of the command-line front end (no GPU work): reconstructs
 * `height` PNG scanlines of `stride` bytes from the inflated image data
 * `raw` (each row: one filter byte, then stride bytes; ISO/IEC 15948
 * section 9) into `out`; bpp = bytes per complete pixel (at least 1).
 * Returns 0, -1 for bad arguments, or r + 1 when row r names an unknown
 * filter.  Replaces the PNG decoding libBICOS's CLI gets from
 * cv::imread (src/fileutils.cpp:61-83). */
int32_t bicos_png_unfilter(uint8_t* out, const uint8_t* raw, int32_t height, size_t stride, int32_t bpp);

/*
 * Frame-by-frame ingest (no counterpart in the reference, whose CLI uploads
 * finished stacks, src/cli.cpp:177-183): a handle owns the device frames of
 * one stack shape.  Each push uploads frame t (0 <= t < n) of both sides
 * from host memory (row step host_step) on `stream` -- asynchronous for
 * pinned memory, so uploads overlap the capture of the next patterns; the
 * host buffers must stay valid until the copy has run.  Pushing a frame
 * again replaces it.  The match runs bicos_match_v1 on the resident frames
 * once every frame has been pushed (BICOS_ERR_EXCEPTION otherwise), ordered
 * after all pushes, on `stream`; outputs as bicos_match_v1.  A handle is
 * used by one host thread at a time; the frames stay resident, so a stack
 * can be matched again (another configuration) without new pushes.
 * Ordering across streams is handled by the handle: matches of one handle
 * run in call order, and a push is ordered after every earlier match, so a
 * capture thread may push the next stack on its upload stream while the
 * previous match still runs on a compute stream.
 */
typedef struct bicos_ingest bicos_ingest;
bicos_status bicos_ingest_create(bicos_ingest** out, int32_t rows, int32_t cols, uint32_t n, int32_t type);
bicos_status bicos_ingest_destroy(bicos_ingest* h);
bicos_status bicos_ingest_push_v1(bicos_ingest* h, uint32_t t, const void* frame0, const void* frame1,
                                  size_t host_step, bicos_stream_t stream);
bicos_status bicos_ingest_match_v1(bicos_ingest* h, bicos_image* disparity, bicos_image* corrmap,
                                   const bicos_config* cfg, bicos_stream_t stream);

/* NCC agreement in place on an int16 disparity; min_var is the per-stack
 * threshold (min_variance * n) used when has_min_var is set. */
bicos_status bicos_agree_v1(bicos_image* disparity, const bicos_image* stack0,
                            const bicos_image* stack1, uint32_t n, float nxcorr_threshold,
                            int32_t has_min_var, float min_var, int32_t precision,
                            bicos_image* corrmap, bicos_stream_t stream);

/* NCC agreement with the subpixel sweep x = -1, -1+step, ... <= 1 (float
 * accumulated); writes a BICOS_32F disparity (NaN = invalid). */
bicos_status bicos_agree_subpixel_v1(const bicos_image* raw_disparity, const bicos_image* stack0,
                                     const bicos_image* stack1, uint32_t n,
                                     float nxcorr_threshold, float subpixel_step,
                                     int32_t has_min_var, float min_var, int32_t precision,
                                     bicos_image* disparity, bicos_image* corrmap,
                                     bicos_stream_t stream);

/*
 * Learned subpixel form (extension; no counterpart in the reference).
 *
 * bicos_subpixel_features_v1: per pixel of a raw int16 disparity, 8 floats
 *   into `features` (float32, rows x 8*cols, 16-byte aligned rows): the
 *   correlation of the left pixel with the right columns col1-2..col1+2
 *   (NaN outside the image), the left and right per-frame variances, and 1
 *   (0 and NaNs for invalid matches).  Exact integer moments (for 8-bit
 *   and 12-bit data, as the MOMENTS form), FP32 ratio.
 * bicos_agree_learned_v1: the LEARNED agreement stage of a raw disparity,
 *   arguments as bicos_agree_subpixel_v1 (min_var already scaled by n);
 *   optionally the network's proposals (float32 image) and, after the
 *   stream completes, the number of pixels that fell back to the sweep.
 * bicos_learned_model_v1: installs a model file image ("BICOSMLP" version
 *   1: header, FP32 input statistics, BF16 parameters) for this process,
 *   replacing the built-in one; NULL uninstalls.  The next learned-form
 *   call on each device uploads it, after synchronising that device when a
 *   previous model is in its buffer (work still in flight, on any stream or
 *   in a cached batch graph, finishes with the model it started with).
 * bicos_mlp_*: the network's own training kernels on device buffers (model
 *   layout: parameters, then 7 input means and 7 standard deviations;
 *   samples: 8 floats, the feature row with the target offset in the last
 *   slot): gradient sum and loss of a batch, an Adam step, and the
 *   proposals of feature rows as the learned form computes them.
 */
bicos_status bicos_subpixel_features_v1(const bicos_image* raw_disparity, const bicos_image* stack0,
                                        const bicos_image* stack1, uint32_t n, bicos_image* features,
                                        bicos_stream_t stream);
bicos_status bicos_agree_learned_v1(const bicos_image* raw_disparity, const bicos_image* stack0,
                                    const bicos_image* stack1, uint32_t n, float nxcorr_threshold,
                                    float subpixel_step, int32_t has_min_var, float min_var, int32_t precision,
                                    bicos_image* disparity, bicos_image* corrmap, bicos_image* proposals,
                                    int32_t* fallback_count, bicos_stream_t stream);
bicos_status bicos_learned_model_v1(const void* data, size_t nbytes);
int bicos_learned_model_installed(void);
bicos_status bicos_learned_model_floats_v1(float* out, int capacity);
void bicos_mlp_sizes(int* n_params, int* n_model_floats);
bicos_status bicos_mlp_grad_v1(const float* model, const float* samples, int count, float* grad, float* loss,
                               void* stream);
bicos_status bicos_mlp_adam_v1(float* params, float* grad, float* m, float* v, int step, float lr,
                               float scale, void* stream);
bicos_status bicos_mlp_propose_v1(const float* model, const float* features, int count, float* out,
                                  void* stream);

/*
 * Batch API (extension; the reference matches one stack per call).
 *
 * A handle owns device workspaces, captured CUDA graphs and a tuning table;
 * it serves one device and one thread at a time.  bicos_match_batch_v1
 * matches `count` items -- each a bicos_match_v1 argument set, stacks of any
 * size, depth, input type and configuration -- in one CUDA graph on
 * `stream`: persistent multi-stack launches for the descriptor transform and
 * the reference-form agreement, the Hamming search per stack on concurrent
 * graph branches.  The graph is captured on the first call with a given
 * signature (shapes, types, configurations, buffer addresses, tuning) and
 * replayed by later calls; each item's results are bit-identical to
 * bicos_match_v1 on the same arguments.  Validation errors name the item
 * ("batch item 3: ...") and launch nothing.  Replays of one graph are
 * ordered on the streams they are issued to.
 *
 * bicos_batch_autotune_v1 times graph replays over the launch shapes
 * (persistent or per-stack launches per stage, transform block width,
 * persistent CTAs per SM, virtual blocks per claim, branches), keeps the
 * fastest for batches of this shape signature
 * (addresses aside) and returns it; results do not depend on the tuning.
 * bicos_batch_set_tuning_v1 fixes a tuning (NULL restores the default and
 * the tuned table); bicos_batch_captures counts graph captures.
 */
typedef struct bicos_batch bicos_batch;

typedef struct bicos_batch_item {
    const bicos_image* stack0;
    const bicos_image* stack1;
    uint32_t n;
    bicos_image* disparity;
    bicos_image* corrmap; /* nullable */
    const bicos_config* cfg;
} bicos_batch_item;

typedef struct bicos_batch_tuning {
    int32_t transform_block; /* 64, 128 or 256 threads (default 256) */
    int32_t ctas_per_sm;     /* persistent launches: CTAs per SM, 1..32 (default 8) */
    int32_t claim;           /* virtual blocks a CTA claims at a time, 1..64 (default 2) */
    int32_t branches;        /* concurrent branches of the per-stack work, 1..4 (default 4) */
    int32_t persistent;      /* bit 0: transform, bit 1: reference-form agreement as persistent
                                multi-stack launches, else per-stack launches on the branches
                                (default 3) */
} bicos_batch_tuning;

bicos_status bicos_batch_create(bicos_batch** out);
bicos_status bicos_batch_destroy(bicos_batch* batch);
bicos_status bicos_match_batch_v1(bicos_batch* batch, const bicos_batch_item* items, uint32_t count,
                                  bicos_stream_t stream);
bicos_status bicos_batch_autotune_v1(bicos_batch* batch, const bicos_batch_item* items, uint32_t count,
                                     bicos_stream_t stream, bicos_batch_tuning* chosen);
bicos_status bicos_batch_get_tuning_v1(const bicos_batch* batch, bicos_batch_tuning* out);
bicos_status bicos_batch_set_tuning_v1(bicos_batch* batch, const bicos_batch_tuning* tuning);
int32_t bicos_batch_captures(const bicos_batch* batch);

/*
 * Stage timing for measurement tools (no counterpart in the reference,
 * whose CLI times whole calls with std::chrono, src/cli.cpp:188-194).  While
 * enabled, each bicos_match_v1 call records CUDA events on its stream
 * around its three stages (descriptor transform, search, agreement), for up
 * to 1024 calls.  bicos_stage_times() waits for those events and returns the
 * summed milliseconds per stage and the number of calls, then starts over.
 */
bicos_status bicos_stage_timing(int32_t enable);
bicos_status bicos_stage_times(float* ms_per_stage /* [3] */, int32_t* calls);

/*
 * FP8 tensor-core rate of the current device for the Hamming search's MMA
 * shape, a measurement tool with no counterpart in the reference: the
 * instruction stream of the search (tcgen05.mma kind::f8f6f4, M = 128,
 * K = 32, four per 128-bit tile) issued alone, two CTAs per SM, timed with
 * CUDA events over three launches.  n = 128 is the search's shape, n = 256
 * the largest single-CTA shape.  *tflops receives 2 x M x N x K per
 * instruction over the time.  Synchronises its own stream; call it when
 * nothing else runs on the device.
 */
bicos_status bicos_tc_fp8_rate_v1(int32_t n, double* tflops);

/* Number of kernel blocks on this device whose bounded waits ran out since
 * load (0 in normal operation; such a block records the event instead of
 * hanging and leaves its outputs unwritten).  Synchronises the device. */
int32_t bicos_kernel_faults(void);

/* Library version string. */
const char* bicos_version(void);

#ifdef __cplusplus
}
#endif

#endif /* BICOS_GB300_C_H */
