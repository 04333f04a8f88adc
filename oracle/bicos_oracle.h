/*
 * CPU oracle for the BICOS matching path.  TEST INFRASTRUCTURE ONLY.
 *
 * This is a plain-C restatement of libBICOS's matching algorithm, used as
 * the checker for the CUDA implementation and as the timed CPU baseline.
 * Nothing in the product library links or calls it.  Each function cites
 * the reference file:line it follows (paths relative to the libBICOS tree).
 *
 * Parity of this restatement is pinned against the reference's own CPU
 * backend (src/impl/cpu.cpp) compiled from source (oracle/ref_build.sh) and
 * against the golden vectors that build produced (tests/golden/).
 *
 * Conventions
 *   - stacks are planar: frame t of a side lives at base + t*rows*cols
 *     elements; elements are uint8 (elem_bytes 1) or uint16 (elem_bytes 2).
 *   - descriptors are arrays of `nwords` uint32 words per pixel, bit i of
 *     the descriptor in word i/32, bit i%32.  On a little-endian machine
 *     this is the byte image of the reference's uint32/uint64/__uint128_t/
 *     std::bitset<256> descriptor types.
 *   - nthreads <= 0 means "all online cores".
 */
#ifndef BICOS_ORACLE_H
#define BICOS_ORACLE_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_OK 0
#define ORC_ERR_EXCEPTION 1        /* reference: BICOS::Exception */
#define ORC_ERR_INVALID_ARGUMENT 2 /* reference: std::invalid_argument */

/* include/impl/common.hpp:46-47 */
#define ORC_FLAG_NODUPES 1
#define ORC_FLAG_CONSISTENCY 2

typedef struct orc_config {
    int32_t has_threshold;
    float nxcorr_threshold;
    int32_t has_subpixel_step;
    float subpixel_step;
    int32_t has_min_variance;
    float min_variance;
    int32_t mode;        /* 0 LIMITED, 1 FULL */
    int32_t precision;   /* 0 SINGLE, 1 DOUBLE */
    int32_t variant;     /* 0 NoDuplicates, 1 Consistency */
    int32_t max_lr_diff;
    int32_t no_dupes;
    int32_t max_bits;    /* 256 = reference limit; up to 512 as an extension */
} orc_config;

int orc_required_bits(int n, int full);
int orc_descriptor_words(int bits, int max_bits);

void orc_transform(const void* stack, int elem_bytes, int n, int rows, int cols,
                   int full, int nwords, uint32_t* out, int nthreads);

void orc_search(const uint32_t* d0, const uint32_t* d1, int rows, int cols,
                int nwords, int flags, int max_lr_diff, int16_t* out,
                int nthreads);

void orc_agree(int16_t* disp, const void* s0, const void* s1, int elem_bytes,
               int n, int rows, int cols, float thr, int has_minvar,
               float minvar, int dbl, void* corrmap, int nthreads);

void orc_agree_subpixel(const int16_t* disp, const void* s0, const void* s1,
                        int elem_bytes, int n, int rows, int cols, float thr,
                        float step, int has_minvar, float minvar, int dbl,
                        float* out, void* corrmap, int nthreads);

float orc_nxcorr_f(const float* x, const float* y, int n, int has_minvar, float minvar);
double orc_nxcorr_d(const double* x, const double* y, int n, int has_minvar, double minvar);

/* Moment form of the agreement stage (the library's extension, no
 * counterpart in the reference): exact integer moments and the closed-form
 * correlation of the unrounded quadratic interpolant, evaluated with the
 * same operations as the CUDA kernel (moments.cu).  mode 0: agree at the
 * integer disparity, out int16 (in place allowed); mode 1: subpixel sweep,
 * out float; mode 2: feature rows, out float[8] per pixel (corr unused).
 * corr: float or double per dbl, may be NULL. */
void orc_moments(const int16_t* disp, const void* s0, const void* s1, int elem_bytes, int n, int rows,
                 int cols, float thr, float step, int has_minvar, float minvar, int dbl, int mode,
                 void* out, void* corr, int nthreads);

/* Learned subpixel form (extension): mode 2 of orc_moments writes the
 * network's feature rows (8 floats per pixel).  orc_learned_check restates
 * the check of the network's proposals: outputs of accepted and border
 * pixels, fallback[px] = 1 where the sweep decides (out/corr untouched). */
void orc_learned_check(const int16_t* disp, const void* s0, const void* s1, int elem_bytes, int n, int rows,
                       int cols, float thr, int has_minvar, float minvar, int dbl, const float* proposal,
                       const float* features, float drop, float* out, void* corrmap, uint8_t* fallback,
                       int nthreads);

/* whole pipeline, src/impl/cpu.cpp:96-155 (+ the CUDA build's precision
 * switch).  disp_out: int16 (no step) or float32 (step); corr_out: float32
 * or float64 per precision, may be NULL.  Returns ORC_* and fills err. */
int orc_match(const void* s0, const void* s1, int elem_bytes, int n, int rows,
              int cols, const orc_config* cfg, void* disp_out, void* corr_out,
              int nthreads, char* err, int errlen);

int orc_num_threads(int nthreads);

#ifdef __cplusplus
}
#endif
#endif
