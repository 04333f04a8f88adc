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

#include "kernels.cuh"

namespace bicos_gb300 {
namespace {

template<typename T>
__device__ __forceinline__ int ld_px(const StackParams& p, int side, int t, int row, int col) {
    const T* r = reinterpret_cast<const T*>(p.frame[side][t] + (long long)row * p.pitch[side][t]);
    return (int)__ldg(r + col);
}

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

template<bool DBL>
struct Prec;
template<>
struct Prec<false> {
    using T = float;
};
template<>
struct Prec<true> {
    using T = double;
};

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
template<typename T, bool DBL, int NMAX>
__global__ void __launch_bounds__(128) k_agree(const __grid_constant__ AgreeParams p) {
    using TP = typename Prec<DBL>::T;
    const int col = blockIdx.x * blockDim.x + threadIdx.x;
    const int row = blockIdx.y;
    const int cols = p.s.cols, n = p.s.n;
    if (col >= cols)
        return;
    int16_t* dp = reinterpret_cast<int16_t*>(reinterpret_cast<char*>(p.raw_io) + row * p.raw_pitch) + col;
    const int16_t d = *dp;
    if (d == kInvalidDisp) {
        put_corr<TP>(p, row, col, (TP)NAN);
        return;
    }
    const int col1 = col - d;
    if (col1 < 0 || cols <= col1) {
        *dp = kInvalidDisp;
        put_corr<TP>(p, row, col, (TP)NAN);
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
    if (nxc < (TP)p.thr)
        *dp = kInvalidDisp;
}

// (T)__float2int_rn(v): round half to even, wrap modulo 2^bits
template<typename T>
__device__ __forceinline__ int round_wrap(float v) {
    return (int)(T)__float2int_rn(v);
}

// agree_subpixel (agree.hpp:94-185, agree.cuh:161-259)
template<typename T, bool DBL, int NMAX>
__global__ void __launch_bounds__(128) k_agree_subpixel(const __grid_constant__ AgreeParams p) {
    using TP = typename Prec<DBL>::T;
    const int col = blockIdx.x * blockDim.x + threadIdx.x;
    const int row = blockIdx.y;
    const int cols = p.s.cols, n = p.s.n;
    if (col >= cols)
        return;
    float result = NAN;
    TP corr = (TP)NAN;
    const int16_t d = reinterpret_cast<const int16_t*>(reinterpret_cast<const char*>(p.raw) + row * p.raw_pitch)[col];
    const int col1 = col - d;
    if (d != kInvalidDisp && col1 >= 0 && col1 < cols) {
        int x[NMAX];
#pragma unroll
        for (int t = 0; t < NMAX; ++t)
            x[t] = t < n ? ld_px<T>(p.s, 0, t, row, col) : 0;
        const bool mv = p.has_minvar != 0;
        if (col1 == 0 || col1 == cols - 1) {
            int y[NMAX];
#pragma unroll
            for (int t = 0; t < NMAX; ++t)
                y[t] = t < n ? ld_px<T>(p.s, 1, t, row, col1) : 0;
            const TP nxc = nxc_full<DBL>(x, y, n, mv, p.minvar);
            corr = nxc;
            if (!(nxc < (TP)p.thr))
                result = (float)d;
        } else {
            float a[NMAX], b[NMAX], c[NMAX];
#pragma unroll
            for (int t = 0; t < NMAX; ++t) {
                if (t < n) {
                    const int y0 = ld_px<T>(p.s, 1, t, row, col1 - 1);
                    const int y1 = ld_px<T>(p.s, 1, t, row, col1);
                    const int y2 = ld_px<T>(p.s, 1, t, row, col1 + 1);
                    // 0.5f*(y0 - 2y1 + y2), 0.5f*(-y0 + y2), y1: exact in float
                    a[t] = 0.5f * (float)(y0 - 2 * y1 + y2);
                    b[t] = 0.5f * (float)(y2 - y0);
                    c[t] = (float)y1;
                } else {
                    a[t] = b[t] = c[t] = 0.f;
                }
            }
            TP d0[NMAX], var0;
            if constexpr (DBL)
                left_d(x, n, d0, var0);
            else
                left_f(x, n, d0, var0);

            float best_x = 0.f;
            TP best = (TP)-1.0;
            for (float xs = -1.f; xs <= 1.f; xs = __fadd_rn(xs, p.step)) {
                int iv[NMAX];
#pragma unroll
                for (int t = 0; t < NMAX; ++t) {
                    const float q = __fadd_rn(__fadd_rn(__fmul_rn(__fmul_rn(a[t], xs), xs), __fmul_rn(b[t], xs)), c[t]);
                    iv[t] = t < n ? round_wrap<T>(q) : 0;
                }
                TP nxc;
                if constexpr (DBL)
                    nxc = nxc_d(d0, var0, iv, n, mv, (double)p.minvar);
                else
                    nxc = nxc_f(d0, var0, iv, n, mv, p.minvar);
                if (best < nxc) {
                    best_x = xs;
                    best = nxc;
                }
            }
            corr = best;
            if (!(best < (TP)p.thr))
                result = __fsub_rn((float)d, best_x);
        }
    }
    reinterpret_cast<float*>(reinterpret_cast<char*>(p.out) + row * p.out_pitch)[col] = result;
    put_corr<TP>(p, row, col, corr);
}

template<typename T, bool DBL, bool SUB>
cudaError_t launch_t(const AgreeParams& p, cudaStream_t st) {
    const dim3 grid((p.s.cols + 127) / 128, p.s.rows);
    const int n = p.s.n;
#define BICOS_AGREE_CASE(NM)                                              \
    if (n <= NM) {                                                        \
        if (SUB)                                                          \
            k_agree_subpixel<T, DBL, NM><<<grid, 128, 0, st>>>(p);        \
        else                                                              \
            k_agree<T, DBL, NM><<<grid, 128, 0, st>>>(p);                 \
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

}  // namespace

cudaError_t launch_agree(const AgreeParams& p, bool dbl, cudaStream_t st) {
    return launch_any<false>(p, dbl, st);
}

cudaError_t launch_agree_subpixel(const AgreeParams& p, bool dbl, cudaStream_t st) {
    return launch_any<true>(p, dbl, st);
}

}  // namespace bicos_gb300
