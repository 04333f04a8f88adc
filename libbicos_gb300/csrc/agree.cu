// NCC agreement and subpixel sweep (stage c).
//
// Semantics: libBICOS include/impl/cpu/agree.hpp:27-185 (float) and
// include/impl/cuda/agree.cuh:35-259 (float nxcorrf / double nxcorrd).
// Every floating-point operation is written with an explicit IEEE
// round-to-nearest intrinsic in the reference's order, so no contraction or
// reassociation can change a threshold decision: the subpixel interpolant is
// ((a*x)*x + b*x) + c with each step rounded, as the reference CPU build
// evaluates it.  Sums of integer samples are exact in float (n*65535 < 2^24)
// and are formed in int.
//
// One thread per pixel; kernels write every output pixel (NaN / INT16_MIN
// where the reference leaves its initial fill), so no separate fill pass
// runs.
#include <math.h>
#include <climits>

#include <type_traits>

#include "batch.cuh"
#include "kernels.cuh"
#include "ncc.cuh"

namespace bicos_gb300 {
namespace {

template<typename TP>
__device__ __forceinline__ void put_corr(const AgreeParams& p, int row, int col, TP v) {
    if (p.corr)
        reinterpret_cast<TP*>(reinterpret_cast<char*>(p.corr) + row * p.corr_pitch)[col] = v;
}

// nxcorrf over integer samples, left statistics precomputed
template<int NMAX>
__device__ __forceinline__ float nxc_f(const float (&d0)[NMAX], float var0, const int (&y)[NMAX], int n,
                                       bool mv, float minvar) {
    int sy = 0;
#pragma unroll
    for (int t = 0; t < NMAX; ++t)
        if (t < n)
            sy += y[t];
    const float m1 = __fdiv_rn((float)sy, (float)n);
    float cov = 0.f, var1 = 0.f;
#pragma unroll
    for (int t = 0; t < NMAX; ++t)
        if (t < n) {
            const float d1 = __fsub_rn((float)y[t], m1);
            cov = __fmaf_rn(d0[t], d1, cov);
            var1 = __fmaf_rn(d1, d1, var1);
        }
    if (mv && (var0 < minvar || var1 < minvar))
        return -1.f;
    return __fdiv_rn(cov, __fsqrt_rn(__fmul_rn(var0, var1)));
}

template<int NMAX>
__device__ __forceinline__ void left_f(const int (&x)[NMAX], int n, float (&d0)[NMAX], float& var0) {
    int sx = 0;
#pragma unroll
    for (int t = 0; t < NMAX; ++t)
        if (t < n)
            sx += x[t];
    const float m0 = __fdiv_rn((float)sx, (float)n);
    var0 = 0.f;
#pragma unroll
    for (int t = 0; t < NMAX; ++t)
        if (t < n) {
            d0[t] = __fsub_rn((float)x[t], m0);
            var0 = __fmaf_rn(d0[t], d0[t], var0);
        }
}

// nxcorrd (include/impl/cuda/agree.cuh:35-65)
template<int NMAX>
__device__ __forceinline__ double nxc_d(const double (&d0)[NMAX], double var0, const int (&y)[NMAX], int n,
                                        bool mv, double minvar) {
    int sy = 0;
#pragma unroll
    for (int t = 0; t < NMAX; ++t)
        if (t < n)
            sy += y[t];
    const double m1 = __ddiv_rn((double)sy, (double)n);
    double cov = 0.0, var1 = 0.0;
#pragma unroll
    for (int t = 0; t < NMAX; ++t)
        if (t < n) {
            const double d1 = __dsub_rn((double)y[t], m1);
            cov = __fma_rn(d0[t], d1, cov);
            var1 = __fma_rn(d1, d1, var1);
        }
    if (mv && (var0 < minvar || var1 < minvar))
        return -1.0;
    return __ddiv_rn(cov, __dsqrt_rn(__dmul_rn(var0, var1)));
}

template<int NMAX>
__device__ __forceinline__ void left_d(const int (&x)[NMAX], int n, double (&d0)[NMAX], double& var0) {
    int sx = 0;
#pragma unroll
    for (int t = 0; t < NMAX; ++t)
        if (t < n)
            sx += x[t];
    const double m0 = __ddiv_rn((double)sx, (double)n);
    var0 = 0.0;
#pragma unroll
    for (int t = 0; t < NMAX; ++t)
        if (t < n) {
            d0[t] = __dsub_rn((double)x[t], m0);
            var0 = __fma_rn(d0[t], d0[t], var0);
        }
}

template<bool DBL, int NMAX>
__device__ __forceinline__ typename Prec<DBL>::T nxc_full(const int (&x)[NMAX], const int (&y)[NMAX], int n,
                                                          bool mv, float minvar) {
    if constexpr (DBL) {
        double d0[NMAX], v0;
        left_d(x, n, d0, v0);
        return nxc_d(d0, v0, y, n, mv, (double)minvar);
    } else {
        float d0[NMAX], v0;
        left_f(x, n, d0, v0);
        return nxc_f(d0, v0, y, n, mv, minvar);
    }
}

// agree, in place on the int16 disparity (agree.hpp:52-92, agree.cuh:110-159)
// Block bodies take the block coordinates as arguments, so the same code
// runs as a grid over one stack and inside a persistent multi-stack launch
// (batch.cuh): bx = column block, row.
template<typename T, bool DBL, int NMAX>
__device__ __forceinline__ void agree_block_body(const AgreeParams& p, int bx, int row) {
    using TP = typename Prec<DBL>::T;
    const int col = bx * blockDim.x + threadIdx.x;
    const int cols = p.s.cols, n = p.s.n;
    if (col >= cols)
        return;
    int16_t* dp = reinterpret_cast<int16_t*>(reinterpret_cast<char*>(p.raw_io) + row * p.raw_pitch) + col;
    const int16_t d = *dp;
    if (d == kInvalidDisp) {
        put_corr<TP>(p, row, col, (TP)NAN);
        agree_point(p, row, col, (float)kInvalidDisp);
        return;
    }
    const int col1 = col - d;
    if (col1 < 0 || cols <= col1) {
        *dp = kInvalidDisp;
        put_corr<TP>(p, row, col, (TP)NAN);
        agree_point(p, row, col, (float)kInvalidDisp);
        return;
    }
    int x[NMAX], y[NMAX];
#pragma unroll
    for (int t = 0; t < NMAX; ++t) {
        x[t] = t < n ? ld_px<T>(p.s, 0, t, row, col) : 0;
        y[t] = t < n ? ld_px<T>(p.s, 1, t, row, col1) : 0;
    }
    const TP nxc = nxc_full<DBL>(x, y, n, p.has_minvar != 0, p.minvar);
    put_corr<TP>(p, row, col, nxc);
    const bool keep = !(nxc < (TP)p.thr);
    if (!keep)
        *dp = kInvalidDisp;
    agree_point(p, row, col, keep ? (float)d : (float)kInvalidDisp);
}

template<typename T, bool DBL, int NMAX>
__global__ void __launch_bounds__(128) k_agree(const __grid_constant__ AgreeParams p) {
    agree_block_body<T, DBL, NMAX>(p, blockIdx.x, blockIdx.y);
}

constexpr int kListThreads = 128;

// The reference sweep (agree.hpp:94-185, agree.cuh:161-259) over the
// pixels of a list, one warp per pixel.  The warp first stages, per frame,
// the interpolation coefficients a, b, c of the right columns col1-1..col1+1
// and the centred left sample d0 = x - mean (position independent, so the
// same values the sequential sweep forms at every position); lane l then
// evaluates positions l, l + 32, ... (xs: the sweep's float-accumulated
// offsets from -1) with the reference's operations in frame order, keeping
// its first strictly better correlation, and the warp keeps the largest at
// its first position -- the offset the sequential sweep keeps.  Sums of
// rounded interpolants are integers below 2^24, exact in float.  Listed
// pixels are interior matches (1 <= col1 <= cols - 2).
template<typename T, bool DBL>
__global__ void __launch_bounds__(kListThreads) k_subpixel_list(const __grid_constant__ AgreeParams p,
                                                                const int* __restrict__ list,
                                                                const int* __restrict__ count,
                                                                const float* __restrict__ xs, int nx) {
    using TP = typename Prec<DBL>::T;
    constexpr int W = kListThreads / 32;
    __shared__ float4 coef_all[W][kMaxFrames];           // a, b, c, d0 (single precision)
    __shared__ double d0_all[DBL ? W : 1][kMaxFrames];  // d0 (double precision)
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    float4* coef = coef_all[w];
    double* d0d = d0_all[DBL ? w : 0];
    const int warp = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    const int nwarps = (int)((gridDim.x * blockDim.x) >> 5);
    const int total = *count, cols = p.s.cols, n = p.s.n;
    const float fn = (float)n;
    const bool mv = p.has_minvar != 0;
    for (int i = warp; i < total; i += nwarps) {
        const int px = list[i];
        const int row = px / cols, col = px - row * cols;
        const int d = reinterpret_cast<const int16_t*>(reinterpret_cast<const char*>(p.raw) + row * p.raw_pitch)[col];
        const int col1 = col - d;
        __syncwarp();  // the previous pixel's coefficients are no longer read
        int xv[3] = {}, sx = 0;
#pragma unroll
        for (int r = 0; r < 3; ++r) {  // frames lane, lane + 32, lane + 64 (n <= 65)
            const int t = lane + 32 * r;
            if (t < n) {
                const int y0 = ld_px<T>(p.s, 1, t, row, col1 - 1);
                const int y1 = ld_px<T>(p.s, 1, t, row, col1);
                const int y2 = ld_px<T>(p.s, 1, t, row, col1 + 1);
                xv[r] = ld_px<T>(p.s, 0, t, row, col);
                sx += xv[r];
                coef[t] = make_float4(0.5f * (float)(y0 - 2 * y1 + y2), 0.5f * (float)(y2 - y0), (float)y1, 0.f);
            }
        }
        sx = __reduce_add_sync(0xffffffffu, sx);  // integer sum: exact in any order
        TP var0 = 0;
        if constexpr (DBL) {
            const double m0 = __ddiv_rn((double)sx, (double)n);
#pragma unroll
            for (int r = 0; r < 3; ++r)
                if (lane + 32 * r < n)
                    d0d[lane + 32 * r] = __dsub_rn((double)xv[r], m0);
            __syncwarp();
            for (int t = 0; t < n; ++t)
                var0 = __fma_rn(d0d[t], d0d[t], var0);
        } else {
            const float m0 = __fdiv_rn((float)sx, fn);
#pragma unroll
            for (int r = 0; r < 3; ++r)
                if (lane + 32 * r < n)
                    coef[lane + 32 * r].w = __fsub_rn((float)xv[r], m0);
            __syncwarp();
            for (int t = 0; t < n; ++t)
                var0 = __fmaf_rn(coef[t].w, coef[t].w, var0);
        }
        TP best = (TP)-1.0;
        int bk = -1;
        for (int k = lane; k < nx; k += 32) {
            const float x = xs[k];
            float sy = 0.f;
#pragma unroll 4
            for (int t = 0; t < n; ++t) {
                const float4 c = coef[t];
                sy = __fadd_rn(sy, round_wrap_f<T>(__fadd_rn(__fadd_rn(__fmul_rn(__fmul_rn(c.x, x), x), __fmul_rn(c.y, x)), c.z)));
            }
            TP cov = 0, var1 = 0, r;
            if constexpr (DBL) {
                const double m1 = __ddiv_rn((double)sy, (double)n);
#pragma unroll 4
                for (int t = 0; t < n; ++t) {
                    const float4 c = coef[t];
                    const float v = round_wrap_f<T>(__fadd_rn(__fadd_rn(__fmul_rn(__fmul_rn(c.x, x), x), __fmul_rn(c.y, x)), c.z));
                    const double d1 = __dsub_rn((double)v, m1);
                    cov = __fma_rn(d0d[t], d1, cov);
                    var1 = __fma_rn(d1, d1, var1);
                }
                r = (mv && (var0 < (double)p.minvar || var1 < (double)p.minvar))
                        ? -1.0 : __ddiv_rn(cov, __dsqrt_rn(__dmul_rn(var0, var1)));
            } else {
                const float m1 = __fdiv_rn(sy, fn);
#pragma unroll 4
                for (int t = 0; t < n; ++t) {
                    const float4 c = coef[t];
                    const float v = round_wrap_f<T>(__fadd_rn(__fadd_rn(__fmul_rn(__fmul_rn(c.x, x), x), __fmul_rn(c.y, x)), c.z));
                    const float d1 = __fsub_rn(v, m1);
                    cov = __fmaf_rn(c.w, d1, cov);
                    var1 = __fmaf_rn(d1, d1, var1);
                }
                r = (mv && (var0 < p.minvar || var1 < p.minvar)) ? -1.f
                                                                   : __fdiv_rn(cov, __fsqrt_rn(__fmul_rn(var0, var1)));
            }
            if (best < r) {
                best = r;
                bk = k;
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const TP ob = __shfl_xor_sync(0xffffffffu, best, o);
            const int ok = __shfl_xor_sync(0xffffffffu, bk, o);
            if (ok >= 0 && (bk < 0 || best < ob || (ob == best && ok < bk))) {
                best = ob;
                bk = ok;
            }
        }
        if (lane == 0) {
            const float bx = bk >= 0 ? xs[bk] : 0.f;
            const float result = !(best < (TP)p.thr) ? __fsub_rn((float)d, bx) : NAN;
            reinterpret_cast<float*>(reinterpret_cast<char*>(p.out) + row * p.out_pitch)[col] = result;
            put_corr<TP>(p, row, col, best);
            agree_point(p, row, col, result);
        }
    }
}

// Single-precision subpixel sweep (agree.hpp:94-185), organised for throughput:
//  - per pixel, the frame coefficients (a, b, c) and the centred left
//    samples d0 are staged once in shared memory as one float4 per frame
//    (each thread reads back only its own column, so no barrier is needed);
//  - XG consecutive sweep points per pass: one coefficient load feeds XG
//    interpolants, the XG covariance chains are independent, and the
//    interpolants stay in registers for the second NCC pass.  Each point's
//    sums still run over t in order, and the best point is taken in
//    increasing x, as the sequential sweep does;
//  - round half to even plus the wrap to T is q + 1.5*2^23 (ulp 1 in
//    [2^23, 2^24)), whose low mantissa bits are the two's-complement
//    integer, masked to 8/16 bits and turned back into a float with the
//    2^23 exponent trick: the value of (T)__float2int_rn(q) without any
//    conversion instruction;
constexpr int kSubThreads = 64;

// Packed FP32 pairs (sm_100+ f32x2 arithmetic): two sweep positions per
// instruction, each lane rounded like the scalar operation (checked one
// operation at a time against the scalar IEEE intrinsics).  A packed
// multiply whose result feeds a packed add is not kept as two roundings by
// the code generator (add.rn/mul.rn notwithstanding; about 40 % of random
// cases came out fused), and neither is fma(t, 1, u) with a literal 1 (it
// is folded into fma(p, q, u) when t = p * q).  So every sum whose operand
// is a product is an explicit fma(t, one, u) with `one` a kernel parameter
// (AgreeParams::one = 1): exact (t * 1 = t) and opaque to the code
// generator.  The interpolant ((a*x)*x + b*x) + c is then three packed
// multiplies and two such FMAs per pair of positions, bit for bit the
// reference's five roundings.
typedef unsigned long long f2;
__device__ __forceinline__ f2 pk(float lo, float hi) {
    f2 r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
    return r;
}
__device__ __forceinline__ void upk(f2 v, float& lo, float& hi) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
}
__device__ __forceinline__ f2 add2(f2 a, f2 b) {
    f2 r;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f2 sub2(f2 a, f2 b) {
    f2 r;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f2 fma2(f2 a, f2 b, f2 c) {
    f2 r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
    return r;
}
__device__ __forceinline__ f2 mul2(f2 a, f2 b) {
    f2 r;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
// ((a*x)*x + b*x) + c on both lanes with the reference's five roundings;
// one = {1, 1} from a kernel parameter
__device__ __forceinline__ f2 interp2(float a, float b, float c, f2 x, f2 one) {
    const f2 t = fma2(mul2(mul2(pk(a, a), x), x), one, mul2(pk(b, b), x));
    return fma2(t, one, pk(c, c));
}
// round_wrap_f on both lanes
template<typename T>
__device__ __forceinline__ f2 round_wrap2(f2 q) {
    constexpr uint32_t kMask = sizeof(T) == 1 ? 0xFFu : 0xFFFFu;
    const f2 f = add2(q, pk(12582912.0f, 12582912.0f));
    uint32_t lo, hi;
    asm("mov.b64 {%0, %1}, %2;" : "=r"(lo), "=r"(hi) : "l"(f));
    lo = (lo & kMask) | 0x4B000000u;
    hi = (hi & kMask) | 0x4B000000u;
    f2 r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "r"(lo), "r"(hi));
    return sub2(r, pk(8388608.0f, 8388608.0f));
}

__device__ __forceinline__ float nxc_from(float cov, float var0, float var1, bool mv, float minvar) {
    return (mv && (var0 < minvar || var1 < minvar)) ? -1.f : __fdiv_rn(cov, __fsqrt_rn(__fmul_rn(var0, var1)));
}

// Smallest frame count of a bucket: every launcher picks the bucket of a
// stack with agree_bucket(n), so n is above the previous bucket's maximum
// and the frame checks below that count fold away at compile time.
__host__ __device__ constexpr int agree_nmin(int nmax) {
    return nmax == 8 ? 1 : nmax == 16 ? 9 : nmax == 24 ? 17 : nmax == 33 ? 25 : nmax == 48 ? 34 : 49;
}

// PREFETCH: request all of a pixel's samples at once (grid launches); the
// persistent multi-stack form streams them, its claim loop leaving no
// registers for the prefetch
template<typename T, int NMAX, bool PREFETCH = true>
__device__ __forceinline__ void subpixel_f32_body(const AgreeParams& p, int bx, int row) {
    constexpr int XG = NMAX <= 33 ? 4 : 2;
    constexpr int kNMin = agree_nmin(NMAX);
    // staged per frame and pixel, as planes: (a, b) pairs, c, d0 (each
    // plane [NMAX][kSubThreads]; 16 bytes per frame and pixel in all) --
    // a thread's reads are consecutive across the warp in every plane, so
    // none conflicts
    extern __shared__ float4 coef_raw[];
    float2* const cab = reinterpret_cast<float2*>(coef_raw);
    float* const cc = reinterpret_cast<float*>(cab + NMAX * kSubThreads);
    float* const cd0 = cc + NMAX * kSubThreads;
    const int tid = threadIdx.x;
    const int col = bx * kSubThreads + tid;
    const int cols = p.s.cols, n = p.s.n;
    if (col >= cols)
        return;
    float result = NAN, corr = NAN;
    const int16_t d = reinterpret_cast<const int16_t*>(reinterpret_cast<const char*>(p.raw) + row * p.raw_pitch)[col];
    const int col1 = col - d;
    const bool mv = p.has_minvar != 0;
    const float fn = (float)n;
    if (d != kInvalidDisp && col1 >= 0 && col1 < cols) {
        const bool border = col1 == 0 || col1 == cols - 1;
        // up to 33 frames, every sample of the pixel is requested at once
        // (the left column and the right triplet of each frame; the border
        // case reads the right column only), so the staging pays one memory
        // latency, not one per few frames; larger stacks (which would not
        // fit in registers) stream the frames, four at a time
        constexpr bool kAll = PREFETCH && NMAX <= 33;
        constexpr int NR = kAll ? NMAX : 1;
        int xl[NR], yl[NR], yc[NR], yr[NR];
        auto sample = [&](int side, int t, int c) { return ld_px<T>(p.s, side, t, row, c); };
        if constexpr (kAll) {
#pragma unroll
            for (int t = 0; t < NMAX; ++t) {
                if (t < kNMin || t < n) {
                    xl[t] = sample(0, t, col);
                    yc[t] = sample(1, t, col1);
                    if (!border) {
                        yl[t] = sample(1, t, col1 - 1);
                        yr[t] = sample(1, t, col1 + 1);
                    }
                }
            }
        }
        auto X = [&](int t) { return kAll ? xl[kAll ? t : 0] : sample(0, t, col); };
        auto YL = [&](int t) { return kAll ? yl[kAll ? t : 0] : sample(1, t, col1 - 1); };
        auto YC = [&](int t) { return kAll ? yc[kAll ? t : 0] : sample(1, t, col1); };
        auto YR = [&](int t) { return kAll ? yr[kAll ? t : 0] : sample(1, t, col1 + 1); };
        int sx = 0, sy = 0;
        if constexpr (kAll) {
#pragma unroll
            for (int t = 0; t < NMAX; ++t)
                if (t < kNMin || t < n) {
                    sx += X(t);
                    sy += YC(t);
                }
        } else {
#pragma unroll 4
            for (int t = 0; t < n; ++t) {
                sx += X(t);
                if (border)
                    sy += YC(t);
            }
        }
        const float m0 = __fdiv_rn((float)sx, fn);
        if (border) {
            const float m1 = __fdiv_rn((float)sy, fn);
            float cov = 0.f, var0 = 0.f, var1 = 0.f;
#pragma unroll
            for (int t = 0; t < NMAX; ++t) {
                if (t < kNMin || t < n) {
                    const float d0 = __fsub_rn((float)X(t), m0);
                    const float d1 = __fsub_rn((float)YC(t), m1);
                    cov = __fmaf_rn(d0, d1, cov);
                    var0 = __fmaf_rn(d0, d0, var0);
                    var1 = __fmaf_rn(d1, d1, var1);
                }
            }
            corr = nxc_from(cov, var0, var1, mv, p.minvar);
            if (!(corr < p.thr))
                result = (float)d;
        } else {
            float var0 = 0.f;
#pragma unroll
            for (int t = 0; t < NMAX; ++t) {
                if (t < kNMin || t < n) {
                    const float d0 = __fsub_rn((float)X(t), m0);
                    var0 = __fmaf_rn(d0, d0, var0);
                    const int y0 = YL(t), y1 = YC(t), y2 = YR(t);
                    cab[t * kSubThreads + tid] = make_float2(0.5f * (float)(y0 - 2 * y1 + y2), 0.5f * (float)(y2 - y0));
                    cc[t * kSubThreads + tid] = (float)y1;
                    cd0[t * kSubThreads + tid] = d0;
                }
            }
            float best_x = 0.f, best = -1.f;
            float xs = -1.f;
            const f2 one2 = pk(p.one, p.one);
            while (xs <= 1.f) {
                float xv[XG];
                bool on[XG];
#pragma unroll
                for (int g = 0; g < XG; ++g) {
                    xv[g] = xs;
                    on[g] = xs <= 1.f;
                    xs = __fadd_rn(xs, p.step);
                }
                constexpr int XP = XG / 2;  // position pairs
                f2 iv[XP][NMAX];
                f2 s1[XP], xq[XP];
#pragma unroll
                for (int q = 0; q < XP; ++q) {
                    s1[q] = 0ull;
                    xq[q] = pk(xv[2 * q], xv[2 * q + 1]);
                }
#pragma unroll
                for (int t = 0; t < NMAX; ++t) {
                    if (t < kNMin || t < n) {
                        const float2 ab = cab[t * kSubThreads + tid];
                        const float c = cc[t * kSubThreads + tid];
#pragma unroll
                        for (int q = 0; q < XP; ++q) {
                            iv[q][t] = round_wrap2<T>(interp2(ab.x, ab.y, c, xq[q], one2));
                            s1[q] = add2(s1[q], iv[q][t]);
                        }
                    }
                    // every fourth frame, a compiler barrier: no coefficient
                    // load is hoisted across it, which bounds the registers
                    // the frame-check-free stretch may take
                    if ((t & 3) == 3)
                        asm volatile("" ::: "memory");
                }
                f2 m1[XP], cov[XP], var1[XP];
#pragma unroll
                for (int q = 0; q < XP; ++q) {
                    float lo, hi;
                    upk(s1[q], lo, hi);
                    m1[q] = pk(__fdiv_rn(lo, fn), __fdiv_rn(hi, fn));
                    cov[q] = 0ull;
                    var1[q] = 0ull;
                }
#pragma unroll
                for (int t = 0; t < NMAX; ++t) {
                    if (t < kNMin || t < n) {
                        const float d0 = cd0[t * kSubThreads + tid];
                        const f2 D0 = pk(d0, d0);
#pragma unroll
                        for (int q = 0; q < XP; ++q) {
                            const f2 d1 = sub2(iv[q][t], m1[q]);
                            cov[q] = fma2(D0, d1, cov[q]);
                            var1[q] = fma2(d1, d1, var1[q]);
                        }
                    }
                    if ((t & 3) == 3)
                        asm volatile("" ::: "memory");
                }
#pragma unroll
                for (int g = 0; g < XG; ++g) {
                    float cv_lo, cv_hi, v1_lo, v1_hi;
                    upk(cov[g / 2], cv_lo, cv_hi);
                    upk(var1[g / 2], v1_lo, v1_hi);
                    const float nxc = nxc_from((g & 1) ? cv_hi : cv_lo, var0, (g & 1) ? v1_hi : v1_lo, mv, p.minvar);
                    if (on[g] && best < nxc) {  // NaN never wins
                        best_x = xv[g];
                        best = nxc;
                    }
                }
            }
            corr = best;
            if (!(best < p.thr))
                result = __fsub_rn((float)d, best_x);
        }
    }
    reinterpret_cast<float*>(reinterpret_cast<char*>(p.out) + row * p.out_pitch)[col] = result;
    put_corr<float>(p, row, col, corr);
    agree_point(p, row, col, result);
}

// six CTAs (12 warps) per SM for the 33-frame bucket: the register cap
// that keeps its sweep within the shared-memory limit's occupancy
template<typename T, int NMAX>
__global__ void __launch_bounds__(kSubThreads, NMAX == 33 ? 6 : 1) k_subpixel_f32(const __grid_constant__ AgreeParams p) {
    subpixel_f32_body<T, NMAX>(p, blockIdx.x, blockIdx.y);
}

// Double-precision subpixel sweep (the reference's nxcorrd,
// include/impl/cuda/agree.cuh:35-65, in agree.cuh:161-259),
// with FP64 work only where it can decide the result:
//  - one pass over the sweep forms, per point, the exact integer moments
//    Sy, Syy, Sxy of the rounded interpolants and an FP32 estimate
//    rho_e = N / sqrt(Dx * Dy)  (N = n Sxy - Sx Sy, D = n S.. - S.^2, all
//    exact integers), whose distance to the reference's FP64 value is below
//    1e-6 (a few FP32 roundings of exact quantities; the FP64 two-pass
//    value differs from the exact correlation by O(n 2^-53));
//  - points whose estimate lies within kWin of the running best are kept
//    (in sweep order), as are points whose min-variance test is too close
//    to call from the exact moments; every other point is provably below
//    the best and cannot be the reference's first maximum;
//  - the kept points are evaluated with the reference's FP64 arithmetic in
//    sweep order.  If more than kKeep points stay kept, the pixel falls
//    back to the FP64 evaluation of every point.
constexpr int kKeep = 6;
constexpr float kWin = 1e-5f;

// (double)v for 0 <= v < 2^31, built with integer instructions (exponent
// from the leading one, the rest of v as the mantissa): exact, and off the
// FP64 pipe, which this kernel keeps busy with the reference's arithmetic
__device__ __forceinline__ double exact_double(int v) {
    const uint32_t u = (uint32_t)v;
    const int e = 31 - __clz(u | 1u);  // v in [2^e, 2^(e+1)) for v > 0
    const unsigned long long mant = ((unsigned long long)u << (52 - e)) & 0xFFFFFFFFFFFFFull;
    const unsigned long long bits = ((unsigned long long)(1023 + e) << 52) | mant;
    return __longlong_as_double(u ? (long long)bits : 0ll);
}

// rounded, wrapped interpolant of sweep point x as an integer: the low
// mantissa bits of q + 1.5*2^23 (see round_wrap_f)
template<typename T>
__device__ __forceinline__ int interp_i(const float4& k, float x) {
    constexpr uint32_t kMask = sizeof(T) == 1 ? 0xFFu : 0xFFFFu;
    const float q = __fadd_rn(__fadd_rn(__fmul_rn(__fmul_rn(k.x, x), x), __fmul_rn(k.y, x)), k.z);
    return (int)(__float_as_uint(__fadd_rn(q, 12582912.0f)) & kMask);
}

// the reference's nxcorrd for sweep point x (left samples, as int bits, in
// coef[].w); sy: the sum of the point's rounded interpolants when the
// screening already has it (exact), else -1
template<typename T, int NMAX>
__device__ double nxcorrd_at(const float4* coef, int tid, int n, double m0, double& var0, bool& have_var0, float x,
                             bool mv, double minvar, long long sy = -1) {
    if (sy < 0) {
        sy = 0;
        for (int t = 0; t < n; ++t)
            sy += interp_i<T>(coef[t * kSubThreads + tid], x);
    }
    const double m1 = __ddiv_rn((double)sy, (double)n);
    double cov = 0.0, var1 = 0.0;
    if (have_var0) {
        for (int t = 0; t < n; ++t) {
            const float4 k = coef[t * kSubThreads + tid];
            const double d0 = __dsub_rn(exact_double(__float_as_int(k.w)), m0);
            const double d1 = __dsub_rn(exact_double(interp_i<T>(k, x)), m1);
            cov = __fma_rn(d0, d1, cov);
            var1 = __fma_rn(d1, d1, var1);
        }
    } else {
        // the first evaluation of a pixel also accumulates the left
        // variance (its own chain, in frame order as before)
        double v0 = 0.0;
        for (int t = 0; t < n; ++t) {
            const float4 k = coef[t * kSubThreads + tid];
            const double d0 = __dsub_rn(exact_double(__float_as_int(k.w)), m0);
            const double d1 = __dsub_rn(exact_double(interp_i<T>(k, x)), m1);
            v0 = __fma_rn(d0, d0, v0);
            cov = __fma_rn(d0, d1, cov);
            var1 = __fma_rn(d1, d1, var1);
        }
        var0 = v0;
        have_var0 = true;
    }
    if (mv && (var0 < minvar || var1 < minvar))
        return -1.0;
    return __ddiv_rn(cov, __dsqrt_rn(__dmul_rn(var0, var1)));
}

template<typename T, int NMAX>
__device__ __forceinline__ void subpixel_f64_body(const AgreeParams& p, int bx, int row) {
    using Acc = typename std::conditional<sizeof(T) == 1, int, long long>::type;
    extern __shared__ float4 coef[];  // [NMAX][kSubThreads]: a, b, c, left sample (int bits)
    const int tid = threadIdx.x;
    const int col = bx * kSubThreads + tid;
    const int cols = p.s.cols, n = p.s.n;
    // every lane of the warp stays to the end: pixels whose kept list
    // overflowed are swept by the whole warp at once
    const bool live = col < cols;
    float result = NAN;
    double corr = NAN;
    const int16_t d = live ? reinterpret_cast<const int16_t*>(reinterpret_cast<const char*>(p.raw) +
                                                              row * p.raw_pitch)[col]
                           : kInvalidDisp;
    const int col1 = col - d;
    bool overflow = false;  // non-border pixel whose kept list overflowed
    double m0_out = 0.0;
    const bool mv = p.has_minvar != 0;
    const double minvar = (double)p.minvar;
    const double dn = (double)n;
    if (d != kInvalidDisp && col1 >= 0 && col1 < cols) {
        long long sx = 0, sxx = 0, sy = 0;
        const bool border = col1 == 0 || col1 == cols - 1;
        // up to 33 frames every sample is requested at once, as in the
        // single-precision sweep; larger stacks stream the frames
        constexpr bool kAll = NMAX <= 33;
        constexpr int NR = kAll ? NMAX : 1;
        int xl[NR], yl[NR], yc[NR], yr[NR];
        auto sample = [&](int side, int t, int c) { return ld_px<T>(p.s, side, t, row, c); };
        if constexpr (kAll) {
#pragma unroll
            for (int t = 0; t < NMAX; ++t) {
                if (t < n) {
                    xl[t] = sample(0, t, col);
                    yc[t] = sample(1, t, col1);
                    if (!border) {
                        yl[t] = sample(1, t, col1 - 1);
                        yr[t] = sample(1, t, col1 + 1);
                    }
                }
            }
        }
        auto X = [&](int t) { return kAll ? xl[kAll ? t : 0] : sample(0, t, col); };
        auto YL = [&](int t) { return kAll ? yl[kAll ? t : 0] : sample(1, t, col1 - 1); };
        auto YC = [&](int t) { return kAll ? yc[kAll ? t : 0] : sample(1, t, col1); };
        auto YR = [&](int t) { return kAll ? yr[kAll ? t : 0] : sample(1, t, col1 + 1); };
#pragma unroll
        for (int t = 0; t < NMAX; ++t) {
            if (t < n) {
                const int x = X(t);
                sx += x;
                sxx += (long long)x * x;
                if (border)
                    sy += YC(t);
            }
        }
        const double m0 = __ddiv_rn((double)sx, dn);
        if (border) {
            const double m1 = __ddiv_rn((double)sy, dn);
            double cov = 0.0, var0 = 0.0, var1 = 0.0;
#pragma unroll
            for (int t = 0; t < NMAX; ++t) {
                if (t < n) {
                    const double d0 = __dsub_rn((double)X(t), m0);
                    const double d1 = __dsub_rn((double)YC(t), m1);
                    cov = __fma_rn(d0, d1, cov);
                    var0 = __fma_rn(d0, d0, var0);
                    var1 = __fma_rn(d1, d1, var1);
                }
            }
            corr = (mv && (var0 < minvar || var1 < minvar)) ? -1.0 : __ddiv_rn(cov, __dsqrt_rn(__dmul_rn(var0, var1)));
            if (!(corr < (double)p.thr))
                result = (float)d;
        } else {
            double var0 = 0.0;  // accumulated by the first FP64 evaluation
            bool have_var0 = false;
#pragma unroll
            for (int t = 0; t < NMAX; ++t) {
                if (t < n) {
                    const int x = X(t);
                    const int y0 = YL(t), y1 = YC(t), y2 = YR(t);
                    coef[t * kSubThreads + tid] =
                        make_float4(0.5f * (float)(y0 - 2 * y1 + y2), 0.5f * (float)(y2 - y0), (float)y1,
                                    __int_as_float(x));
                }
            }
            // exact left moment and its min-variance decision
            const long long dx = (long long)n * sxx - sx * sx;  // n^2 * variance
            const Acc dxa = (Acc)dx;
            const double mvn = minvar * dn;                    // exact
            // the min-variance decisions in integers, thresholds made once:
            // dd < mvn <=> dd < ceil(mvn); the FP64 reference may decide
            // otherwise only within 1e-9 (relative) of mvn, the band
            // [ceil(mvn - tol), floor(mvn + tol)]
            const double tol = 1e-9 * fmax(mvn, 1.0);
            auto to_ll = [](double v) -> long long {
                return v >= 9.0e18 ? LLONG_MAX : v <= -9.0e18 ? LLONG_MIN : (long long)v;
            };
            const long long cmv = to_ll(ceil(mvn)), ulo = to_ll(ceil(mvn - tol)), uhi = to_ll(floor(mvn + tol));
            auto below = [&](long long dd, bool& unsure) {
                unsure = dd >= ulo && dd <= uhi;
                return dd < cmv;
            };
            bool unsure0;
            const bool low0 = mv && below(dx, unsure0);
            unsure0 = mv && unsure0;

            float keep_x[kKeep];
            float keep_r[kKeep];
            bool keep_f[kKeep];
            long long keep_s[kKeep];
            int nk = 0;
            float best_e = -1.f;  // running best estimate (the sweep starts at -1)
            float xs = -1.f;
            const f2 one2 = pk(p.one, p.one);
            constexpr uint32_t kMask = sizeof(T) == 1 ? 0xFFu : 0xFFFFu;
            // two sweep points per pass on packed FP32 pairs (the same
            // roundings as interp_i), their moments in exact integers
            while (xs <= 1.f) {
                float xv[2];
                bool on[2];
#pragma unroll
                for (int g = 0; g < 2; ++g) {
                    xv[g] = xs;
                    on[g] = xs <= 1.f;
                    xs = __fadd_rn(xs, p.step);
                }
                const f2 xq = pk(xv[0], xv[1]);
                Acc s1[2] = {0, 0}, s11[2] = {0, 0}, s01[2] = {0, 0};
                for (int t = 0; t < n; ++t) {
                    const float4 k = coef[t * kSubThreads + tid];
                    const f2 f = add2(interp2(k.x, k.y, k.z, xq, one2), pk(12582912.0f, 12582912.0f));
                    uint32_t lo, hi;
                    asm("mov.b64 {%0, %1}, %2;" : "=r"(lo), "=r"(hi) : "l"(f));
                    const Acc va = (Acc)(lo & kMask), vb = (Acc)(hi & kMask), xi = (Acc)__float_as_int(k.w);
                    s1[0] += va;
                    s11[0] += va * va;
                    s01[0] += xi * va;
                    s1[1] += vb;
                    s11[1] += vb * vb;
                    s01[1] += xi * vb;
                }
#pragma unroll
                for (int g = 0; g < 2; ++g) {
                    if (!on[g])
                        continue;
                    // 8-bit samples: every moment below fits in 32 bits
                    // (n <= 65: n * sum y^2 < 2^31), so the conversions to
                    // float are the 32-bit ones
                    const Acc S1 = s1[g], S11 = s11[g], S01 = s01[g];
                    const Acc dy = (Acc)n * S11 - S1 * S1;
                    const Acc num = (Acc)n * S01 - (Acc)sx * S1;
                    bool unsure1 = false;
                    const bool low1 = mv && below(dy, unsure1);
                    unsure1 = mv && unsure1;
                    float re;
                    if (low0 || low1)
                        re = -1.f;
                    else
                        re = (float)num * rsqrtf((float)dxa * (float)dy);  // NaN when flat
                    const bool forced = unsure0 || unsure1;
                    if (forced || re >= best_e - kWin) {
                        if (re > best_e) {
                            // drop kept points that fell out of the window
                            int w = 0;
                            for (int i = 0; i < nk; ++i)
                                if (keep_f[i] || keep_r[i] >= re - kWin) {
                                    keep_x[w] = keep_x[i];
                                    keep_r[w] = keep_r[i];
                                    keep_f[w] = keep_f[i];
                                    keep_s[w] = keep_s[i];
                                    ++w;
                                }
                            nk = w;
                            if (!forced)
                                best_e = re;
                        }
                        if (nk < kKeep) {
                            keep_x[nk] = xv[g];
                            keep_r[nk] = re;
                            keep_f[nk] = forced;
                            keep_s[nk] = S1;
                            ++nk;
                        } else {
                            overflow = true;
                        }
                    }
                }
            }

            double best = -1.0;
            float best_x = 0.f;
            if (!overflow) {
                for (int i = 0; i < nk; ++i) {
                    if (!keep_f[i] && keep_r[i] < best_e - kWin)
                        continue;
                    const double r =
                        nxcorrd_at<T, NMAX>(coef, tid, n, m0, var0, have_var0, keep_x[i], mv, minvar, keep_s[i]);
                    if (best < r) {
                        best = r;
                        best_x = keep_x[i];
                    }
                }
                corr = best;
                if (!(best < (double)p.thr))
                    result = __fsub_rn((float)d, best_x);
            } else {
                m0_out = m0;  // swept below by the whole warp
            }
        }
    }
    // Pixels whose kept list overflowed: every sweep point evaluated with
    // the reference's FP64 arithmetic, one point per lane of the warp, and
    // the first maximum taken across lanes in sweep order (the sequential
    // sweep's `best < r` keeps the first of equal maxima, starts from -1
    // and never takes NaN).  Each lane computes the pixel's left variance
    // along the way (the same chain, so the same value).
    unsigned ovf = __ballot_sync(0xffffffffu, overflow);
    const int lane = tid & 31, wbase = tid & ~31;
    if (ovf)
        __syncwarp();  // the swept pixel's staged coefficients, visible to the warp
    while (ovf) {
        const int src = __ffs(ovf) - 1;
        ovf &= ovf - 1;
        const double m0s = __shfl_sync(0xffffffffu, m0_out, src);
        double best = -1.0;
        float best_x = 0.f;
        float xc = -1.f;  // first sweep point of this chunk of 32
        bool more = true;
        while (more) {
            float x = xc;
            for (int k = 0; k < lane; ++k)
                x = __fadd_rn(x, p.step);
            double r = -INFINITY;
            if (x <= 1.f) {
                double v0 = 0.0;
                bool hv0 = false;
                r = nxcorrd_at<T, NMAX>(coef, wbase + src, n, m0s, v0, hv0, x, mv, minvar);
                if (!(r > -1.0))
                    r = -INFINITY;  // cannot beat the initial -1 (or NaN)
            }
            // first maximum across the chunk: larger r, then smaller lane
            double rb = r;
            int lb = lane;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const double ro = __shfl_xor_sync(0xffffffffu, rb, o);
                const int lo = __shfl_xor_sync(0xffffffffu, lb, o);
                if (ro > rb || (ro == rb && lo < lb)) {
                    rb = ro;
                    lb = lo;
                }
            }
            const float xb = __shfl_sync(0xffffffffu, x, lb);
            if (best < rb) {  // chunks in sweep order
                best = rb;
                best_x = xb;
            }
            // the next chunk starts after the chunk's last point
            const float xl = __shfl_sync(0xffffffffu, x, 31);
            xc = __fadd_rn(xl, p.step);
            more = xl <= 1.f && xc <= 1.f;
        }
        if (lane == src) {
            corr = best;
            if (!(best < (double)p.thr))
                result = __fsub_rn((float)d, best_x);
        }
        __syncwarp();  // reads of the staged column done before it is reused
    }
    if (!live)
        return;
    reinterpret_cast<float*>(reinterpret_cast<char*>(p.out) + row * p.out_pitch)[col] = result;
    put_corr<double>(p, row, col, corr);
    agree_point(p, row, col, result);
}

template<typename T, int NMAX>
__global__ void __launch_bounds__(kSubThreads) k_subpixel_f64(const __grid_constant__ AgreeParams p) {
    subpixel_f64_body<T, NMAX>(p, blockIdx.x, blockIdx.y);
}

// persistent multi-stack forms (batch.cuh)
template<typename T, bool DBL, int NMAX>
struct AgreeOp {
    using P = AgreeParams;
    static constexpr int kMaxThreads = 128;
    static constexpr int kMinBlocks = 1;
    static __device__ __forceinline__ void run(const P& p, int bx, int row, int) {
        agree_block_body<T, DBL, NMAX>(p, bx, row);
    }
};
template<typename T, int NMAX>
struct SubF32Op {
    using P = AgreeParams;
    static constexpr int kMaxThreads = kSubThreads;
    static constexpr int kMinBlocks = 1;
    static __device__ __forceinline__ void run(const P& p, int bx, int row, int) {
        subpixel_f32_body<T, NMAX, false>(p, bx, row);
    }
};
template<typename T, int NMAX>
struct SubF64Op {
    using P = AgreeParams;
    static constexpr int kMaxThreads = kSubThreads;
    static constexpr int kMinBlocks = 1;
    static __device__ __forceinline__ void run(const P& p, int bx, int row, int) {
        subpixel_f64_body<T, NMAX>(p, bx, row);
    }
};

// the sweep's offsets: -1, then float additions of the step while <= 1
__global__ void k_sweep_offsets(float step, float* __restrict__ xs, int nx) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        int k = 0;
        for (float x = -1.f; x <= 1.f && k < nx; x = __fadd_rn(x, step))
            xs[k++] = x;
    }
}

template<typename T, int NM>
cudaError_t launch_subpixel_f64(const AgreeParams& p, cudaStream_t st) {
    const size_t smem = (size_t)NM * kSubThreads * sizeof(float4);
    auto k = k_subpixel_f64<T, NM>;
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess)
            return e;
    }
    const dim3 grid((p.s.cols + kSubThreads - 1) / kSubThreads, p.s.rows);
    k<<<grid, kSubThreads, smem, st>>>(p);
    return cudaGetLastError();
}

template<typename T, int NM>
cudaError_t launch_subpixel_f32(const AgreeParams& p, cudaStream_t st) {
    const size_t smem = (size_t)NM * kSubThreads * sizeof(float4);
    auto k = k_subpixel_f32<T, NM>;
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess)
            return e;
    }
    const dim3 grid((p.s.cols + kSubThreads - 1) / kSubThreads, p.s.rows);
    k<<<grid, kSubThreads, smem, st>>>(p);
    return cudaGetLastError();
}

template<typename T, bool DBL, bool SUB>
cudaError_t launch_t(const AgreeParams& p, cudaStream_t st) {
    const dim3 grid((p.s.cols + 127) / 128, p.s.rows);
    const int n = p.s.n;
#define BICOS_AGREE_CASE(NM)                                         \
    if (n <= NM) {                                                        \
        if (SUB && !DBL)                                                  \
            return launch_subpixel_f32<T, NM>(p, st);                     \
        if (SUB)                                                          \
            return launch_subpixel_f64<T, NM>(p, st);                     \
        k_agree<T, DBL, NM><<<grid, 128, 0, st>>>(p);                     \
        return cudaGetLastError();                                        \
    }
    BICOS_AGREE_CASE(8)
    BICOS_AGREE_CASE(16)
    BICOS_AGREE_CASE(24)
    BICOS_AGREE_CASE(33)
    BICOS_AGREE_CASE(48)
    BICOS_AGREE_CASE(65)
#undef BICOS_AGREE_CASE
    return cudaErrorInvalidValue;
}

template<bool SUB>
cudaError_t launch_any(const AgreeParams& p, bool dbl, cudaStream_t st) {
    if (p.s.elem_bytes == 1)
        return dbl ? launch_t<uint8_t, true, SUB>(p, st) : launch_t<uint8_t, false, SUB>(p, st);
    return dbl ? launch_t<uint16_t, true, SUB>(p, st) : launch_t<uint16_t, false, SUB>(p, st);
}

template<typename T, bool DBL>
cudaError_t launch_list_t(const AgreeParams& p, const int* list, const int* count, const float* xs, int nx,
                          cudaStream_t st) {
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess)
        e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess)
        return e;
    // grid-stride over a list whose length only the device knows
    k_subpixel_list<T, DBL><<<sms * 16, kListThreads, 0, st>>>(p, list, count, xs, nx);
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_subpixel_list(const AgreeParams& p, bool dbl, const int* list, const int* count,
                                 const float* xs, int nx, cudaStream_t st) {
    if (p.s.elem_bytes == 1)
        return dbl ? launch_list_t<uint8_t, true>(p, list, count, xs, nx, st)
                   : launch_list_t<uint8_t, false>(p, list, count, xs, nx, st);
    return dbl ? launch_list_t<uint16_t, true>(p, list, count, xs, nx, st)
               : launch_list_t<uint16_t, false>(p, list, count, xs, nx, st);
}

namespace {
template<typename T, int NM>
cudaError_t agree_batch_nm(int kind, bool dbl, const BatchArgs<AgreeParams>& a, const BatchLaunch& l,
                           cudaStream_t st) {
    if (kind == 1)
        return launch_batch_op<SubF32Op<T, NM>>(a, l, agree_smem(1, NM), st);
    if (kind == 2)
        return launch_batch_op<SubF64Op<T, NM>>(a, l, agree_smem(2, NM), st);
    return dbl ? launch_batch_op<AgreeOp<T, true, NM>>(a, l, 0, st)
               : launch_batch_op<AgreeOp<T, false, NM>>(a, l, 0, st);
}

template<typename T>
cudaError_t agree_batch_t(int kind, bool dbl, int nmax, const BatchArgs<AgreeParams>& a, const BatchLaunch& l,
                          cudaStream_t st) {
    switch (nmax) {
        case 8: return agree_batch_nm<T, 8>(kind, dbl, a, l, st);
        case 16: return agree_batch_nm<T, 16>(kind, dbl, a, l, st);
        case 24: return agree_batch_nm<T, 24>(kind, dbl, a, l, st);
        case 33: return agree_batch_nm<T, 33>(kind, dbl, a, l, st);
        case 48: return agree_batch_nm<T, 48>(kind, dbl, a, l, st);
        case 65: return agree_batch_nm<T, 65>(kind, dbl, a, l, st);
        default: return cudaErrorInvalidValue;
    }
}
}  // namespace

int agree_bucket(int n) {
    for (int b : {8, 16, 24, 33, 48, 65})
        if (n <= b)
            return b;
    return -1;
}

int agree_block(int kind) { return kind == 0 ? 128 : kSubThreads; }

size_t agree_smem(int kind, int nmax) { return kind == 0 ? 0 : (size_t)nmax * kSubThreads * sizeof(float4); }

cudaError_t launch_agree_batch(int elem_bytes, int kind, bool dbl, int nmax, const BatchArgs<AgreeParams>& a,
                               const BatchLaunch& l, cudaStream_t st) {
    return elem_bytes == 1 ? agree_batch_t<uint8_t>(kind, dbl, nmax, a, l, st)
                           : agree_batch_t<uint16_t>(kind, dbl, nmax, a, l, st);
}

int sweep_offset_count(float step) {
    int k = 0;
    for (float x = -1.f; x <= 1.f; x += step)
        ++k;
    return k;
}

cudaError_t launch_sweep_offsets(float step, float* xs, int nx, cudaStream_t st) {
    k_sweep_offsets<<<1, 32, 0, st>>>(step, xs, nx);
    return cudaGetLastError();
}

cudaError_t launch_agree(const AgreeParams& p, bool dbl, cudaStream_t st) {
    return launch_any<false>(p, dbl, st);
}

cudaError_t launch_agree_subpixel(const AgreeParams& p, bool dbl, cudaStream_t st) {
    return launch_any<true>(p, dbl, st);
}

}  // namespace bicos_gb300
