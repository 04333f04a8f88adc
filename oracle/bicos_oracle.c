/*
 * CPU oracle for the BICOS matching path.  TEST INFRASTRUCTURE ONLY: the
 * checker for the CUDA implementation and the timed CPU baseline ("port").
 * The product library never links, loads or calls this file.
 *
 * A plain-C restatement of libBICOS 2.2.0's CPU backend.  Every function
 * names the reference file:line it follows.  The double-precision NCC
 * follows the reference CUDA backend (the CPU backend computes only in
 * float).  Build with -ffp-contract=off: the subpixel interpolant
 * a*x*x + b*x + c must round after every operation, as the reference CPU
 * build on x86-64 does.
 */
#define _GNU_SOURCE
#include "bicos_oracle.h"

#include <limits.h>
#include <math.h>
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

#define INVALID_I16 ((int16_t)INT16_MIN) /* include/common.hpp:34-37 */
#define INVALID_INT INT_MIN

int orc_num_threads(int nthreads) {
    if (nthreads > 0)
        return nthreads;
    long c = sysconf(_SC_NPROCESSORS_ONLN);
    return c > 0 ? (int)c : 1;
}

/* ---- row-parallel driver (stands in for cv::parallel_for_) ---- */

typedef void (*row_fn)(void* ctx, int row_begin, int row_end);

typedef struct {
    row_fn fn;
    void* ctx;
    int begin, end;
} row_job;

static void* row_job_run(void* p) {
    row_job* j = (row_job*)p;
    j->fn(j->ctx, j->begin, j->end);
    return NULL;
}

static void parallel_rows(int rows, int nthreads, row_fn fn, void* ctx) {
    int nt = orc_num_threads(nthreads);
    if (nt > rows)
        nt = rows;
    if (nt <= 1) {
        fn(ctx, 0, rows);
        return;
    }
    pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * nt);
    row_job* jobs = (row_job*)malloc(sizeof(row_job) * nt);
    for (int i = 0; i < nt; ++i) {
        jobs[i].fn = fn;
        jobs[i].ctx = ctx;
        jobs[i].begin = (int)((long)rows * i / nt);
        jobs[i].end = (int)((long)rows * (i + 1) / nt);
        pthread_create(&th[i], NULL, row_job_run, &jobs[i]);
    }
    for (int i = 0; i < nt; ++i)
        pthread_join(th[i], NULL);
    free(th);
    free(jobs);
}

static inline int load_px(const void* base, int elem_bytes, size_t idx) {
    return elem_bytes == 1 ? (int)((const uint8_t*)base)[idx] : (int)((const uint16_t*)base)[idx];
}

/* ---- descriptor bits (include/impl/cpu/bitfield.hpp:34-58: LSB first) ---- */

typedef struct {
    uint32_t* w;
    int i;
} bitsink;

static inline void bs_set(bitsink* b, int v) {
    if (v)
        b->w[b->i >> 5] |= 1u << (b->i & 31);
    b->i++;
}

/* include/impl/cpu/descriptor_transform.hpp:31-73 */
static void transform_limited_px(const int* pix, int n, bitsink* bf) {
    float av = 0.0f;
    for (int t = 0; t < n; ++t)
        av += (float)pix[t];
    av /= (float)n;

    int prev[2] = {-1, -1};
    for (int t = 0; t < n - 2; ++t) {
        const int a = pix[t], b = pix[t + 1], c = pix[t + 2];
        bs_set(bf, a < b);
        bs_set(bf, a < c);
        bs_set(bf, (float)a < av);
        const int cur = a + b;
        if (prev[t % 2] != -1)
            bs_set(bf, prev[t % 2] < cur);
        prev[t % 2] = cur;
    }
    const int a = pix[n - 2], b = pix[n - 1];
    bs_set(bf, a < b);
    bs_set(bf, (float)a < av);
    bs_set(bf, (float)b < av);
    bs_set(bf, prev[(n - 2) % 2] < a + b);
}

/* include/impl/cpu/descriptor_transform.hpp:75-123 */
static void transform_full_px(const int* pix, int n, bitsink* bf) {
    float av = 0.0f;
    for (int t = 0; t < n; ++t)
        av += (float)pix[t];
    av /= (float)n;

    int pairsums[130];
    for (int t = 0; t < n - 2; ++t) {
        const int a = pix[t], b = pix[t + 1], c = pix[t + 2];
        bs_set(bf, a < b);
        bs_set(bf, a < c);
        bs_set(bf, (float)a < av);
        pairsums[t] = pix[t] + pix[t + 1];
    }
    pairsums[n - 2] = pix[n - 2] + pix[n - 1];
    const int a = pix[n - 2], b = pix[n - 1];
    bs_set(bf, a < b);
    bs_set(bf, (float)a < av);
    bs_set(bf, (float)b < av);
    for (int t = 0; t < n - 1; ++t)
        for (int i = 0; i < n - 1; ++i) {
            if (i == t || i == t - 1 || i == t + 1)
                continue;
            bs_set(bf, pairsums[t] < pairsums[i]);
        }
}

typedef struct {
    const void* stack;
    int elem_bytes, n, rows, cols, full, nwords;
    uint32_t* out;
} tf_ctx;

/* include/impl/cpu/descriptor_transform.hpp:125-138 */
static void transform_rows(void* p, int r0, int r1) {
    tf_ctx* c = (tf_ctx*)p;
    const size_t plane = (size_t)c->rows * c->cols;
    int pix[130];
    for (int r = r0; r < r1; ++r)
        for (int col = 0; col < c->cols; ++col) {
            const size_t px = (size_t)r * c->cols + col;
            for (int t = 0; t < c->n; ++t)
                pix[t] = load_px(c->stack, c->elem_bytes, (size_t)t * plane + px);
            uint32_t* w = c->out + px * c->nwords;
            memset(w, 0, sizeof(uint32_t) * c->nwords);
            bitsink bf = {w, 0};
            if (c->full)
                transform_full_px(pix, c->n, &bf);
            else
                transform_limited_px(pix, c->n, &bf);
        }
}

void orc_transform(const void* stack, int elem_bytes, int n, int rows, int cols,
                   int full, int nwords, uint32_t* out, int nthreads) {
    tf_ctx c = {stack, elem_bytes, n, rows, cols, full, nwords, out};
    parallel_rows(rows, nthreads, transform_rows, &c);
}

/* ---- Hamming arg-min, include/impl/cpu/bicos.hpp:29-76 ---- */

static inline int ham(const uint32_t* a, const uint32_t* b, int nwords) {
    int s = 0;
    for (int k = 0; k < nwords; ++k)
        s += __builtin_popcount(a[k] ^ b[k]);
    return s;
}

/* 64-bit popcounts over pairs of words (the reference's u64/u128 words,
 * include/impl/cpu/bicos.hpp:29-48); same counts as ham() */
static inline int ham64(const uint32_t* a, const uint32_t* b, int npairs) {
    int s = 0;
    for (int k = 0; k < npairs; ++k) {
        uint64_t x, y;
        memcpy(&x, a + 2 * k, 8);
        memcpy(&y, b + 2 * k, 8);
        s += __builtin_popcountll(x ^ y);
    }
    return s;
}

/* include/impl/cpu/bicos.hpp:50-76; one body per descriptor width so the
 * word loop is unrolled (the reference's template on the descriptor type) */
#define ORC_SEARCH_BODY(COST)                                                \
    int best = INVALID_INT, min_cost = INT_MAX, dups = 0;                  \
    for (int c1 = 0; c1 < cols; ++c1) {                                    \
        const uint32_t* cand = row1 + (size_t)c1 * nwords;                 \
        const int cost = (COST);                                           \
        if (cost < min_cost) {                                             \
            min_cost = cost;                                               \
            best = c1;                                                     \
            if (flags & ORC_FLAG_NODUPES)                                  \
                dups = 0;                                                  \
        } else if ((flags & ORC_FLAG_NODUPES) && cost == min_cost)         \
            dups++;                                                        \
    }                                                                      \
    if ((flags & ORC_FLAG_NODUPES) && dups > 0)                            \
        return INVALID_INT;                                                \
    return best;

#define ORC_SEARCH_NW(NAME, NPAIRS)                                                       \
    static int NAME(const uint32_t* d0, const uint32_t* row1, int cols, int flags) {     \
        const int nwords = 2 * (NPAIRS);                                                  \
        ORC_SEARCH_BODY(ham64(d0, cand, NPAIRS))                                          \
    }
ORC_SEARCH_NW(search_w2, 1)
ORC_SEARCH_NW(search_w4, 2)
ORC_SEARCH_NW(search_w8, 4)
ORC_SEARCH_NW(search_w12, 6)
ORC_SEARCH_NW(search_w16, 8)

static int search_any(const uint32_t* d0, const uint32_t* row1, int cols, int nwords, int flags) {
    ORC_SEARCH_BODY(ham(d0, cand, nwords))
}

static int bicos_search(const uint32_t* d0, const uint32_t* row1, int cols, int nwords, int flags) {
    switch (nwords) {
        case 2: return search_w2(d0, row1, cols, flags);
        case 4: return search_w4(d0, row1, cols, flags);
        case 8: return search_w8(d0, row1, cols, flags);
        case 12: return search_w12(d0, row1, cols, flags);
        case 16: return search_w16(d0, row1, cols, flags);
        default: return search_any(d0, row1, cols, nwords, flags);
    }
}

typedef struct {
    const uint32_t *d0, *d1;
    int rows, cols, nwords, flags, max_lr_diff;
    int16_t* out;
} search_ctx;

/* include/impl/cpu/bicos.hpp:78-113 */
static void search_rows(void* p, int r0, int r1) {
    search_ctx* c = (search_ctx*)p;
    const size_t rstride = (size_t)c->cols * c->nwords;
    for (int r = r0; r < r1; ++r) {
        const uint32_t* row0 = c->d0 + r * rstride;
        const uint32_t* row1 = c->d1 + r * rstride;
        int16_t* o = c->out + (size_t)r * c->cols;
        for (int c0 = 0; c0 < c->cols; ++c0) {
            o[c0] = INVALID_I16;
            const int best = bicos_search(row0 + (size_t)c0 * c->nwords, row1, c->cols, c->nwords, c->flags);
            if (best == INVALID_INT)
                continue;
            if (c->flags & ORC_FLAG_CONSISTENCY) {
                const int rev = bicos_search(row1 + (size_t)best * c->nwords, row0, c->cols, c->nwords, c->flags);
                if (rev == INVALID_INT || abs(c0 - rev) > c->max_lr_diff)
                    continue;
                o[c0] = (int16_t)((c0 + rev) / 2 - best);
            } else
                o[c0] = (int16_t)(c0 - best);
        }
    }
}

void orc_search(const uint32_t* d0, const uint32_t* d1, int rows, int cols, int nwords,
                int flags, int max_lr_diff, int16_t* out, int nthreads) {
    search_ctx c = {d0, d1, rows, cols, nwords, flags, max_lr_diff, out};
    parallel_rows(rows, nthreads, search_rows, &c);
}

/* ---- NCC ---- */

/* include/impl/cpu/agree.hpp:27-50 (float, the CPU backend's only form;
 * identical arithmetic to nxcorrf, include/impl/cuda/agree.cuh:67-97) */
float orc_nxcorr_f(const float* x, const float* y, int n, int has_minvar, float minvar) {
    float mean0 = 0.f, mean1 = 0.f;
    for (int i = 0; i < n; ++i) {
        mean0 += x[i];
        mean1 += y[i];
    }
    mean0 /= (float)n;
    mean1 /= (float)n;
    float covar = 0.f, var0 = 0.f, var1 = 0.f;
    for (int i = 0; i < n; ++i) {
        const float d0 = x[i] - mean0, d1 = y[i] - mean1;
        covar = fmaf(d0, d1, covar);
        var0 = fmaf(d0, d0, var0);
        var1 = fmaf(d1, d1, var1);
    }
    if (has_minvar && (var0 < minvar || var1 < minvar))
        return -1.f;
    return covar / sqrtf(var0 * var1);
}

/* include/impl/cuda/agree.cuh:35-65 (nxcorrd; no CPU counterpart) */
double orc_nxcorr_d(const double* x, const double* y, int n, int has_minvar, double minvar) {
    double mean0 = 0.0, mean1 = 0.0;
    for (int i = 0; i < n; ++i) {
        mean0 += x[i];
        mean1 += y[i];
    }
    mean0 /= (double)n;
    mean1 /= (double)n;
    double covar = 0.0, var0 = 0.0, var1 = 0.0;
    for (int i = 0; i < n; ++i) {
        const double d0 = x[i] - mean0, d1 = y[i] - mean1;
        covar = fma(d0, d1, covar);
        var0 = fma(d0, d0, var0);
        var1 = fma(d1, d1, var1);
    }
    if (has_minvar && (var0 < minvar || var1 < minvar))
        return -1.0;
    return covar / sqrt(var0 * var1);
}

typedef struct {
    int16_t* disp_io;     /* agree: in place */
    const int16_t* disp;  /* subpixel: read only */
    const void *s0, *s1;
    int elem_bytes, n, rows, cols;
    float thr, step;
    int has_minvar;
    float minvar;
    int dbl;
    float* out;
    void* corr;
    /* learned-form check */
    const float* proposal;
    const float* features;
    float drop;
    uint8_t* fallback;
} agree_ctx;

static inline void put_corr(agree_ctx* c, size_t px, double v) {
    if (!c->corr)
        return;
    if (c->dbl)
        ((double*)c->corr)[px] = v;
    else
        ((float*)c->corr)[px] = (float)v;
}

static double nxc_px(agree_ctx* c, const int* x, const int* y) {
    if (c->dbl) {
        double xd[130], yd[130];
        for (int t = 0; t < c->n; ++t) {
            xd[t] = x[t];
            yd[t] = y[t];
        }
        return orc_nxcorr_d(xd, yd, c->n, c->has_minvar, (double)c->minvar);
    }
    float xf[130], yf[130];
    for (int t = 0; t < c->n; ++t) {
        xf[t] = (float)x[t];
        yf[t] = (float)y[t];
    }
    return orc_nxcorr_f(xf, yf, c->n, c->has_minvar, c->minvar);
}

/* threshold test in the working precision: float, or double against the
 * float threshold widened (src/impl/cuda.cu.in:223, agree.cuh:156) */
static inline int below(agree_ctx* c, double nxc) {
    if (c->dbl)
        return nxc < (double)c->thr;
    return (float)nxc < c->thr;
}

/* include/impl/cpu/agree.hpp:52-92 */
static void agree_rows(void* p, int r0, int r1) {
    agree_ctx* c = (agree_ctx*)p;
    const size_t plane = (size_t)c->rows * c->cols;
    int x[130], y[130];
    for (int r = r0; r < r1; ++r)
        for (int col = 0; col < c->cols; ++col) {
            const size_t px = (size_t)r * c->cols + col;
            int16_t* d = c->disp_io + px;
            if (*d == INVALID_I16)
                continue;
            const int idx1 = col - *d;
            if (idx1 < 0 || c->cols <= idx1) {
                *d = INVALID_I16;
                continue;
            }
            const size_t px1 = (size_t)r * c->cols + idx1;
            for (int t = 0; t < c->n; ++t) {
                x[t] = load_px(c->s0, c->elem_bytes, t * plane + px);
                y[t] = load_px(c->s1, c->elem_bytes, t * plane + px1);
            }
            const double nxc = nxc_px(c, x, y);
            put_corr(c, px, nxc);
            if (below(c, nxc))
                *d = INVALID_I16;
        }
}

void orc_agree(int16_t* disp, const void* s0, const void* s1, int elem_bytes, int n,
               int rows, int cols, float thr, int has_minvar, float minvar, int dbl,
               void* corrmap, int nthreads) {
    agree_ctx c;
    memset(&c, 0, sizeof c);
    c.disp_io = disp;
    c.s0 = s0;
    c.s1 = s1;
    c.elem_bytes = elem_bytes;
    c.n = n;
    c.rows = rows;
    c.cols = cols;
    c.thr = thr;
    c.has_minvar = has_minvar;
    c.minvar = minvar;
    c.dbl = dbl;
    c.corr = corrmap;
    parallel_rows(rows, nthreads, agree_rows, &c);
}

/* (TInput)roundevenf(v) as the reference's x86-64 build evaluates it (and as
 * the CUDA backend's (TInput)__float2int_rn(v) does): round half to even,
 * then wrap modulo 2^bits.  Written via int so it is defined on every host. */
static inline int round_wrap(float v, int elem_bytes) {
    const int r = (int)rintf(v);
    return elem_bytes == 1 ? (int)(uint8_t)r : (int)(uint16_t)r;
}

/* include/impl/cpu/agree.hpp:94-185 (double form: agree.cuh:161-259) */
static void subpixel_rows(void* p, int r0, int r1) {
    agree_ctx* c = (agree_ctx*)p;
    const size_t plane = (size_t)c->rows * c->cols;
    const int n = c->n;
    int x[130], y[130], interp[130];
    float a[130], b[130], cc[130];
    for (int r = r0; r < r1; ++r)
        for (int col = 0; col < c->cols; ++col) {
            const size_t px = (size_t)r * c->cols + col;
            const int16_t d = c->disp[px];
            if (d == INVALID_I16)
                continue;
            const int col1 = col - d;
            if (col1 < 0 || c->cols <= col1)
                continue;
            for (int t = 0; t < n; ++t)
                x[t] = load_px(c->s0, c->elem_bytes, t * plane + px);
            const size_t row1 = (size_t)r * c->cols;
            if (col1 == 0 || col1 == c->cols - 1) {
                for (int t = 0; t < n; ++t)
                    y[t] = load_px(c->s1, c->elem_bytes, t * plane + row1 + col1);
                const double nxc = nxc_px(c, x, y);
                put_corr(c, px, nxc);
                if (below(c, nxc))
                    continue;
                c->out[px] = (float)d;
                continue;
            }
            for (int t = 0; t < n; ++t) {
                const int y0 = load_px(c->s1, c->elem_bytes, t * plane + row1 + col1 - 1);
                const int y1 = load_px(c->s1, c->elem_bytes, t * plane + row1 + col1);
                const int y2 = load_px(c->s1, c->elem_bytes, t * plane + row1 + col1 + 1);
                a[t] = 0.5f * ((float)y0 - 2.0f * (float)y1 + (float)y2);
                b[t] = 0.5f * (float)(-y0 + y2);
                cc[t] = (float)y1;
            }
            float best_x = 0.f;
            double best = -1.0;
            for (float xs = -1.f; xs <= 1.f; xs += c->step) {
                for (int t = 0; t < n; ++t)
                    interp[t] = round_wrap(a[t] * xs * xs + b[t] * xs + cc[t], c->elem_bytes);
                const double nxc = nxc_px(c, x, interp);
                const int better = c->dbl ? (best < nxc) : ((float)best < (float)nxc);
                if (better) {
                    best_x = xs;
                    best = nxc;
                }
            }
            put_corr(c, px, best);
            if (below(c, best))
                continue;
            c->out[px] = (float)d - best_x;
        }
}

void orc_agree_subpixel(const int16_t* disp, const void* s0, const void* s1, int elem_bytes,
                        int n, int rows, int cols, float thr, float step, int has_minvar,
                        float minvar, int dbl, float* out, void* corrmap, int nthreads) {
    const size_t px = (size_t)rows * cols;
    for (size_t i = 0; i < px; ++i)
        out[i] = NAN;
    agree_ctx c;
    memset(&c, 0, sizeof c);
    c.disp = disp;
    c.s0 = s0;
    c.s1 = s1;
    c.elem_bytes = elem_bytes;
    c.n = n;
    c.rows = rows;
    c.cols = cols;
    c.thr = thr;
    c.step = step;
    c.has_minvar = has_minvar;
    c.minvar = minvar;
    c.dbl = dbl;
    c.out = out;
    c.corr = corrmap;
    parallel_rows(rows, nthreads, subpixel_rows, &c);
}

/* Learned form's check (the library's extension; restates agree.cu's
 * k_learned_check): border pixels as the sweep; elsewhere one reference NCC
 * at the proposed offset, accepted when rho(x) >= rho(0) - drop with rho(0)
 * the feature row's integer-disparity correlation; rejected pixels are
 * flagged for the sweep and left unwritten. */
static void learned_rows(void* p, int r0, int r1) {
    agree_ctx* c = (agree_ctx*)p;
    const size_t plane = (size_t)c->rows * c->cols;
    const int n = c->n;
    int x[130], y[130], interp[130];
    for (int r = r0; r < r1; ++r)
        for (int col = 0; col < c->cols; ++col) {
            const size_t px = (size_t)r * c->cols + col;
            c->fallback[px] = 0;
            const int16_t d = c->disp[px];
            if (d == INVALID_I16)
                continue;
            const int col1 = col - d;
            if (col1 < 0 || c->cols <= col1)
                continue;
            for (int t = 0; t < n; ++t)
                x[t] = load_px(c->s0, c->elem_bytes, t * plane + px);
            const size_t row1 = (size_t)r * c->cols;
            if (col1 == 0 || col1 == c->cols - 1) {
                for (int t = 0; t < n; ++t)
                    y[t] = load_px(c->s1, c->elem_bytes, t * plane + row1 + col1);
                const double nxc = nxc_px(c, x, y);
                put_corr(c, px, nxc);
                if (!below(c, nxc))
                    c->out[px] = (float)d;
                continue;
            }
            const float xo = c->proposal[px];
            for (int t = 0; t < n; ++t) {
                const int y0 = load_px(c->s1, c->elem_bytes, t * plane + row1 + col1 - 1);
                const int y1 = load_px(c->s1, c->elem_bytes, t * plane + row1 + col1);
                const int y2 = load_px(c->s1, c->elem_bytes, t * plane + row1 + col1 + 1);
                const float a = 0.5f * ((float)y0 - 2.0f * (float)y1 + (float)y2);
                const float b = 0.5f * (float)(-y0 + y2);
                interp[t] = round_wrap(a * xo * xo + b * xo + (float)y1, c->elem_bytes);
            }
            const double nxc = nxc_px(c, x, interp);
            const float r0f = c->features[8 * px + 2];
            const double floor_rho = c->dbl ? (double)r0f - (double)c->drop : (double)(r0f - c->drop);
            if (!(nxc >= floor_rho)) {
                c->fallback[px] = 1;
                continue;
            }
            put_corr(c, px, nxc);
            if (!below(c, nxc))
                c->out[px] = (float)d - xo;
        }
}

void orc_learned_check(const int16_t* disp, const void* s0, const void* s1, int elem_bytes, int n, int rows,
                       int cols, float thr, int has_minvar, float minvar, int dbl, const float* proposal,
                       const float* features, float drop, float* out, void* corrmap, uint8_t* fallback,
                       int nthreads) {
    const size_t px = (size_t)rows * cols;
    for (size_t i = 0; i < px; ++i)
        out[i] = NAN;
    agree_ctx c;
    memset(&c, 0, sizeof c);
    c.disp = disp;
    c.s0 = s0;
    c.s1 = s1;
    c.elem_bytes = elem_bytes;
    c.n = n;
    c.rows = rows;
    c.cols = cols;
    c.thr = thr;
    c.has_minvar = has_minvar;
    c.minvar = minvar;
    c.dbl = dbl;
    c.out = out;
    c.corr = corrmap;
    c.proposal = proposal;
    c.features = features;
    c.drop = drop;
    c.fallback = fallback;
    parallel_rows(rows, nthreads, learned_rows, &c);
}

/* ---- dispatch, src/impl/cpu.cpp:96-155 ---- */

int orc_required_bits(int n, int full) {
    return full ? n * n - 2 * n + 3 : 4 * n - 7;
}

/* src/impl/cpu.cpp:125-152: uint32 / uint64 / uint128 / bitset<256>.  Past
 * 256 bits (an extension, only when max_bits allows) the width rounds up
 * to a multiple of 128 bits. */
int orc_descriptor_words(int bits, int max_bits) {
    if (bits <= 32)
        return 1;
    if (bits <= 64)
        return 2;
    if (bits <= 128)
        return 4;
    if (bits <= 256)
        return 8;
    if (bits <= max_bits && bits <= 512)
        return ((bits + 127) / 128) * 4;
    return -1;
}

int orc_match(const void* s0, const void* s1, int elem_bytes, int n, int rows, int cols,
              const orc_config* cfg, void* disp_out, void* corr_out, int nthreads,
              char* err, int errlen) {
    if (n < 2) {
        snprintf(err, errlen, "need at least two images");
        return ORC_ERR_EXCEPTION;
    }
    if (elem_bytes != 1 && elem_bytes != 2) {
        snprintf(err, errlen, "bad input depths, only CV_8UC1 and CV_16UC1 are supported");
        return ORC_ERR_EXCEPTION;
    }
    const int bits = orc_required_bits(n, cfg->mode == 1);
    const int nwords = orc_descriptor_words(bits, cfg->max_bits > 256 ? cfg->max_bits : 256);
    if (nwords < 0) {
        snprintf(err, errlen, "input stacks too large, would require %d bits", bits);
        return ORC_ERR_INVALID_ARGUMENT;
    }
    if (cfg->has_threshold && cfg->has_subpixel_step && !(cfg->subpixel_step >= 1e-4f)) {
        snprintf(err, errlen, "subpixel step must be at least 1e-4");
        return ORC_ERR_EXCEPTION;
    }
    const float minvar = cfg->has_min_variance ? cfg->min_variance * (float)n : 0.f;
    const size_t px = (size_t)rows * cols;
    uint32_t* d0 = (uint32_t*)calloc(px * nwords, sizeof(uint32_t));
    uint32_t* d1 = (uint32_t*)calloc(px * nwords, sizeof(uint32_t));
    orc_transform(s0, elem_bytes, n, rows, cols, cfg->mode == 1, nwords, d0, nthreads);
    orc_transform(s1, elem_bytes, n, rows, cols, cfg->mode == 1, nwords, d1, nthreads);

    int flags;
    int lr = -1;
    if (cfg->variant == 1) {
        flags = ORC_FLAG_CONSISTENCY | (cfg->no_dupes ? ORC_FLAG_NODUPES : 0);
        lr = cfg->max_lr_diff;
    } else
        flags = ORC_FLAG_NODUPES;

    const int subpix = cfg->has_threshold && cfg->has_subpixel_step;
    int16_t* raw = subpix ? (int16_t*)malloc(px * sizeof(int16_t)) : (int16_t*)disp_out;
    orc_search(d0, d1, rows, cols, nwords, flags, lr, raw, nthreads);
    free(d0);
    free(d1);

    if (cfg->has_threshold) {
        const int dbl = cfg->precision == 1;
        if (corr_out) {
            for (size_t i = 0; i < px; ++i) {
                if (dbl)
                    ((double*)corr_out)[i] = NAN;
                else
                    ((float*)corr_out)[i] = NAN;
            }
        }
        if (subpix) {
            orc_agree_subpixel(raw, s0, s1, elem_bytes, n, rows, cols, cfg->nxcorr_threshold,
                               cfg->subpixel_step, cfg->has_min_variance, minvar, dbl,
                               (float*)disp_out, corr_out, nthreads);
            free(raw);
        } else
            orc_agree(raw, s0, s1, elem_bytes, n, rows, cols, cfg->nxcorr_threshold,
                      cfg->has_min_variance, minvar, dbl, corr_out, nthreads);
    }
    return ORC_OK;
}

/* ---- moment form (the library's extension; restates moments.cu) ---- */

typedef struct {
    const int16_t* disp;
    const void *s0, *s1;
    int elem_bytes, n, rows, cols;
    float thr, step;
    int has_minvar;
    float minvar;
    int dbl, mode;
    void* out;
    void* corr;
} mom_ctx;

/* correlation ratio p / sqrt(v0 * q), rounded as in the kernel */
static double mom_ratio(int dbl, double p, double v0, double q) {
    if (dbl)
        return p / sqrt(v0 * q);
    return (double)((float)p / sqrtf((float)v0 * (float)q));
}

static double mom_fma(int dbl, double a, double b, double c) {
    return dbl ? fma(a, b, c) : (double)fmaf((float)a, (float)b, (float)c);
}

/* conversion of an exact int64 to the working precision */
static double mom_cvt(int dbl, long long v) {
    return dbl ? (double)v : (double)(float)v;
}

static void moments_rows(void* p, int r0, int r1) {
    mom_ctx* c = (mom_ctx*)p;
    const size_t plane = (size_t)c->rows * c->cols;
    const long long nn = c->n;
    for (int r = r0; r < r1; ++r)
        for (int col = 0; col < c->cols; ++col) {
            const size_t px = (size_t)r * c->cols + col;
            const int16_t d = c->disp[px];
            const int col1 = col - d;
            const int valid = d != INVALID_I16 && col1 >= 0 && col1 < c->cols;
            double corr = NAN;
            float fout = NAN;
            int16_t iout = INVALID_I16;
            if (valid) {
                long long sx = 0, sxx = 0, sy[5] = {0}, sxy[5] = {0}, syy[5][5] = {{0}};
                for (int t = 0; t < c->n; ++t) {
                    const long long x = load_px(c->s0, c->elem_bytes, t * plane + px);
                    long long y[5];
                    sx += x;
                    sxx += x * x;
                    for (int j = 0; j < 5; ++j) {
                        const int cc = col1 + j - 2;
                        y[j] = (cc >= 0 && cc < c->cols) ? load_px(c->s1, c->elem_bytes, t * plane + (size_t)r * c->cols + cc) : 0;
                        sy[j] += y[j];
                        sxy[j] += x * y[j];
                    }
                    for (int j = 0; j < 5; ++j)
                        for (int k = j; k < 5; ++k)
                            syy[j][k] += y[j] * y[k];
                }
                const long long v0 = nn * sxx - sx * sx;
                if (c->mode == 2) {
                    /* learned-form features: rho at col1-2..col1+2 (FP32
                     * ratio, NaN outside the image), variances, flag */
                    float* f = (float*)c->out + 8 * px;
                    for (int j = 0; j < 5; ++j) {
                        const int cc = col1 + j - 2;
                        if (cc >= 0 && cc < c->cols) {
                            const long long v1 = nn * syy[j][j] - sy[j] * sy[j];
                            f[j] = (float)mom_ratio(0, mom_cvt(0, nn * sxy[j] - sx * sy[j]), mom_cvt(0, v0),
                                                    mom_cvt(0, v1));
                        } else {
                            f[j] = NAN;
                        }
                    }
                    const float n2 = (float)c->n * (float)c->n;
                    f[5] = (float)v0 / n2;
                    f[6] = (float)(nn * syy[2][2] - sy[2] * sy[2]) / n2;
                    f[7] = 1.f;
                    continue;
                }
                const double mvn = c->dbl ? (double)c->minvar * (double)c->n
                                          : (double)((float)c->minvar * (float)c->n);
                const double V0 = mom_cvt(c->dbl, v0);
                const int low0 = c->has_minvar && V0 < mvn;
                const int border = col1 == 0 || col1 == c->cols - 1;
                if (c->mode == 0 || border) {
                    const long long v1 = nn * syy[2][2] - sy[2] * sy[2];
                    const double V1 = mom_cvt(c->dbl, v1);
                    if (c->has_minvar && (low0 || V1 < mvn))
                        corr = -1.0;
                    else
                        corr = mom_ratio(c->dbl, mom_cvt(c->dbl, nn * sxy[2] - sx * sy[2]), V0, V1);
                    const int pass = !(c->dbl ? corr < (double)c->thr : (float)corr < c->thr);
                    if (pass) {
                        iout = d;
                        fout = (float)d;
                    }
                } else {
                    const long long XA = sxy[1] - 2 * sxy[2] + sxy[3], XB = sxy[3] - sxy[1], XC = sxy[2];
                    const long long YA = sy[1] - 2 * sy[2] + sy[3], YB = sy[3] - sy[1], YC = sy[2];
                    const long long Smm = syy[1][1], Szz = syy[2][2], Sqq = syy[3][3], Smz = syy[1][2],
                                    Szq = syy[2][3], Smq = syy[1][3];
                    const long long AA = Smm + 4 * Szz + Sqq - 4 * Smz - 4 * Szq + 2 * Smq;
                    const long long AB = Sqq - Smm + 2 * Smz - 2 * Szq;
                    const long long BB = Sqq - 2 * Smq + Smm;
                    const long long AC2 = Smz - 2 * Szz + Szq;
                    const long long BC2 = Szq - Smz;
                    const long long CC = Szz;
                    const int D = c->dbl;
                    const double P2 = mom_cvt(D, nn * XA - sx * YA), P1 = mom_cvt(D, nn * XB - sx * YB),
                                 P0 = mom_cvt(D, 2 * (nn * XC - sx * YC));
                    const double Q4 = mom_cvt(D, nn * AA - YA * YA), Q3 = mom_cvt(D, 2 * (nn * AB - YA * YB)),
                                 Q2 = mom_cvt(D, nn * BB + 4 * nn * AC2 - YB * YB - 4 * YA * YC),
                                 Q1 = mom_cvt(D, 4 * (nn * BC2 - YB * YC)), Q0 = mom_cvt(D, 4 * (nn * CC - YC * YC));
                    const double mvq = D ? 4.0 * mvn : (double)(4.0f * (float)mvn);
                    double best = -1.0;
                    float best_x = 0.f;
                    for (float xs = -1.f; xs <= 1.f; xs += c->step) {
                        const double X = xs;
                        const double Pv = mom_fma(D, mom_fma(D, P2, X, P1), X, P0);
                        const double Qv = mom_fma(D, mom_fma(D, mom_fma(D, mom_fma(D, Q4, X, Q3), X, Q2), X, Q1), X, Q0);
                        const double rr = (low0 || (c->has_minvar && Qv < mvq)) ? -1.0 : mom_ratio(D, Pv, V0, Qv);
                        const int better = D ? best < rr : (float)best < (float)rr;
                        if (better) {
                            best = rr;
                            best_x = xs;
                        }
                    }
                    corr = best;
                    const int pass = !(D ? best < (double)c->thr : (float)best < c->thr);
                    if (pass)
                        fout = (float)d - best_x;
                }
            }
            if (c->mode == 2) {
                float* f = (float*)c->out + 8 * px;
                for (int j = 0; j < 7; ++j)
                    f[j] = NAN;
                f[7] = 0.f;
                continue;
            }
            if (c->mode == 0)
                ((int16_t*)c->out)[px] = iout;
            else
                ((float*)c->out)[px] = fout;
            if (c->corr) {
                if (c->dbl)
                    ((double*)c->corr)[px] = corr;
                else
                    ((float*)c->corr)[px] = (float)corr;
            }
        }
}

void orc_moments(const int16_t* disp, const void* s0, const void* s1, int elem_bytes, int n, int rows, int cols,
                 float thr, float step, int has_minvar, float minvar, int dbl, int mode, void* out, void* corr,
                 int nthreads) {
    mom_ctx c = {disp, s0, s1, elem_bytes, n, rows, cols, thr, step, has_minvar, minvar, dbl, mode, out, corr};
    if (mode == 0 && out == (void*)disp) {
        /* in place: work from a copy of the input disparity */
        const size_t px = (size_t)rows * cols;
        int16_t* copy = (int16_t*)malloc(px * sizeof(int16_t));
        memcpy(copy, disp, px * sizeof(int16_t));
        c.disp = copy;
        parallel_rows(rows, nthreads, moments_rows, &c);
        free(copy);
        return;
    }
    parallel_rows(rows, nthreads, moments_rows, &c);
}
